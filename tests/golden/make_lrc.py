"""Golden values of the reference's homogeneous long-range correction
(longRange/Homogeneous: UpotCorr and VirialCorr), computed by the
reference itself through oracle/ref/ref_harness.cpp's `lrc` mode, for LJ
(centred, shifted), the 2CLJQ/1CLJD mixture (off-centre LJ sites, dipole
self term) and two of the reference's own test inputs.  Writes lrc_*.npz in
the format of make_golden.py (phase space + rc) plus upot_corr, virial_corr.

    python tests/golden/make_lrc.py [--ref /path/to/ls1-mardyn]
"""
import argparse
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402


def run_lrc(path, rc, rclj):
    p = mg.subprocess.run([mg.HARNESS, "lrc", path, str(rc), str(rclj)], capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stderr[-2000:])
    for line in p.stdout.splitlines():
        t = line.split()
        if t and t[0] == "LRC":
            return float(t[1]), float(t[2])
    raise RuntimeError("no LRC record")


def store(name, ps, rc, rclj, u, w):
    d = dict(box=ps.box, components=mg.components_json(ps), mixing=np.array(ps.mixing).reshape(-1, 2),
             eps_rf=ps.eps_rf, ids=ps.ids, comp=ps.comp, r=ps.r, v=ps.v, q=ps.q, L=ps.L, rc=rc, rc_lj=rclj,
             periodic=1, upot_corr=u, virial_corr=w)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"{name}: N={ps.n} UpotCorr={u!r} VirialCorr={w!r}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    a = ap.parse_args()
    if a.ref is None:
        sys.path.insert(0, mg.ROOT)
        from oracle.refpath import reference_tree
        a.ref = reference_tree()
    tmp = tempfile.mkdtemp()
    cases = [("lj864", mg.psm.lj_fcc(6, 0.7, 1.1, seed=3), 2.5, 2.5),
             ("lj864_shifted", mg.psm.lj_fcc(6, 0.7, 1.1, seed=3, shifted=True, rc=2.5), 2.5, 2.5),
             ("lj864_rclj", mg.psm.lj_fcc(6, 0.7, 1.1, seed=3), 3.0, 2.2),
             ("mix500", mg.psm.mixture(500, 18.0, 300.0, seed=31), 1.0, 1.0)]
    for name, ps, rc, rclj in cases:
        path = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, path)
        ps = mg.psm.read_inp(path)
        store("lrc_" + name, ps, rc, rclj, *run_lrc(path, rc, rclj))
    tin = os.path.join(a.ref, "test_input")
    for name, rc in (("VectorizationWater", 6.16), ("VectorizationMultiComponentMultiPotentials", 35.0)):
        path = os.path.join(tin, name + ".inp")
        ps = mg.psm.read_inp(path)
        store("lrc_ref_" + name, ps, rc, rc, *run_lrc(path, rc, rc))


if __name__ == "__main__":
    main()
