"""Golden runs of the reference's planar long-range correction
(longRange/Planar) driven by oracle/ref/ref_harness.cpp's `planar` mode:
NVE steps with Planar::calculateLongRange between the traversal and calcFM
(at the first force evaluation and in every step).  Writes planar_*.npz in
the format of make_golden.py plus the per-call corrections (lrc: UpotCorr,
VirialCorr), the slab settings and the target temperature.

    python tests/golden/make_planar.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402


def yslab(cells_xy, seed):
    """The vapour-liquid slab generator's box with its normal turned from z to y."""
    ps = mg.psm.lj_slab(cells_xy, 0.73, 0.02, 0.9, seed=seed)
    ps.r = ps.r[:, [0, 2, 1]].copy()
    ps.v = ps.v[:, [0, 2, 1]].copy()
    ps.box = ps.box[[0, 2, 1]].copy()
    ps.temperature = 0.9
    return ps


def dipolar_first_mixture(n, seed):
    """The 2CLJQ/1CLJD mixture with the dipolar component first (the
    reference indexes its squared net dipoles by component index, which is
    only well defined when the dipolar components come first)."""
    ps = mg.psm.mixture(n, 18.0, 300.0, seed=seed)
    ps.components = ps.components[::-1]
    ps.comp = (1 - ps.comp).astype(np.int32)
    ps.temperature = 300.0
    return ps


def main():
    tmp = tempfile.mkdtemp()
    # name, phase space, rc, dt, steps, slabs, frequency, region as fractions of L_y
    cases = [("slab1clj", yslab(6, 7), 3.0, 0.002, 6, 200, 3, (0.0, 1.0)),
             ("slab1clj_region", yslab(6, 8), 3.0, 0.002, 4, 150, 2, (0.3, 0.7)),
             ("mix500", dipolar_first_mixture(500, 31), 1.0, 9.118e-5, 3, 40, 2, (0.0, 1.0))]
    for name, ps, rc, dt, n, slabs, freq, reg in cases:
        path = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, path)
        T = ps.temperature
        ps = mg.psm.read_inp(path)
        lo, hi = float(reg[0] * ps.box[1]), float(reg[1] * ps.box[1])
        p = mg.subprocess.run([mg.HARNESS, "planar", path, str(rc), str(rc), str(dt), str(n), str(slabs), str(freq),
                               repr(float(lo)), repr(float(hi))], capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-2000:])
        res = mg.parse(p.stdout)
        res["grid"] = np.zeros(3, np.int64)
        res["cell_length"] = np.zeros(3)
        mg.store("planar_" + name, ps, rc, rc, True, res, dt, n, True)
        z = dict(np.load(os.path.join(HERE, "planar_" + name + ".npz")))
        z["lrc"] = np.array([[float(x) for x in l.split()[1:]] for l in p.stdout.splitlines() if l.startswith("LRC")])
        z["slabs"], z["frequency"] = slabs, freq
        z["region"] = np.array([lo, hi])
        z["target_temperature"] = T
        np.savez_compressed(os.path.join(HERE, "planar_" + name + ".npz"), **z)


if __name__ == "__main__":
    main()
