"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference implementation's short-range path (built from its own
sources by ``oracle/ref/Makefile`` into ``oracle/_ref/``) on
  * the reference's own unit-test inputs for this path
    (test_input/ForceCalculationTest{U0,F0}.inp with cut-offs 1.1 / 1.3 and the
    ten test_input/Vectorization*.inp files with the cut-offs of
    src/particleContainer/adapter/tests/VectorizedCellProcessorTest.cpp:136-388),
    set up without halo exactly as those tests do, and
  * seeded periodic cases written by ``ls1gb300.phasespace`` (LJ fcc with
    jitter, LJ with a separate LJ cut-off and shifted potential, the 2CLJQ/1CLJD
    mixture with reaction field, a vapour-liquid slab, and the 1CLJ N=32000 case
    over 100 Leapfrog steps),
and stores inputs and outputs as ``.npz``.  Only this script reads the
reference tree; the fixtures travel with the repository.

    python tests/golden/make_golden.py [--ref <ls1-mardyn tree>]   (default: oracle/refpath.py)
"""
import argparse
import dataclasses
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
from ls1gb300 import phasespace as psm  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness_DPDP")


def components_json(ps):
    return json.dumps([dataclasses.asdict(c) for c in ps.components])


def parse(out: str):
    res = {"mol": [], "steps": []}
    for line in out.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "GRID":
            res["grid"] = np.array([int(x) for x in t[1:4]])
            res["cell_length"] = np.array([float(x) for x in t[4:7]])
        elif t[0] == "UPOT":
            res["upot"] = float(t[1])
        elif t[0] == "VIRIAL":
            res["virial"] = float(t[1])
        elif t[0] == "COUNTS":
            res["counts"] = np.array([float(x) for x in t[1:]])
        elif t[0] == "STEP":
            res["steps"].append([float(x) for x in t[1:]])
        elif t[0] == "MOL":
            res["mol"].append([float(x) for x in t[1:]])
    return res


def run(args):
    p = subprocess.run([HARNESS] + [str(a) for a in args], capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"harness failed: {args}\n{p.stderr[-2000:]}")
    return parse(p.stdout)


def store(name, ps, rc, rclj, periodic, res, dt=0.0, nsteps=0, keep_molecules=True):
    mol = np.array(res["mol"])
    d = dict(box=ps.box, components=components_json(ps), mixing=np.array(ps.mixing).reshape(-1, 2),
             eps_rf=ps.eps_rf, ids=ps.ids, comp=ps.comp, r=ps.r, v=ps.v, q=ps.q, L=ps.L,
             rc=rc, rc_lj=rclj, periodic=int(periodic), dt=dt, nsteps=nsteps,
             grid=res["grid"], cell_length=res["cell_length"])
    if "upot" in res:
        d.update(upot=res["upot"], virial=res["virial"], counts=res["counts"])
    if res["steps"]:
        d["steps"] = np.array(res["steps"])
    if keep_molecules:
        d.update(out_ids=mol[:, 0].astype(np.uint64), out_comp=mol[:, 1].astype(np.int32),
                 out_cell=mol[:, 2].astype(np.int64), out_r=mol[:, 3:6], out_v=mol[:, 6:9],
                 out_q=mol[:, 9:13], out_L=mol[:, 13:16], F=mol[:, 16:19], M=mol[:, 19:22], Vi=mol[:, 22:25])
    else:
        d.update(out_n=mol.shape[0], out_r_sum=mol[:, 3:6].sum(axis=0), out_v_sum=mol[:, 6:9].sum(axis=0))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"{name}: N={ps.n} out={mol.shape[0]} upot={res.get('upot', res['steps'][-1][1] if res['steps'] else None)}")


def jitter(ps, amp, seed):
    rng = np.random.default_rng(seed)
    ps.r = ps.r + rng.uniform(-amp, amp, ps.r.shape)
    return ps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    a = ap.parse_args()
    if a.ref is None:
        sys.path.insert(0, ROOT)
        from oracle.refpath import reference_tree
        a.ref = reference_tree()
    tin = os.path.join(a.ref, "test_input")
    tmp = tempfile.mkdtemp()

    # (1) the reference's own unit-test inputs, set up without halo as its tests do
    cases = [("ForceCalculationTestU0", 1.1), ("ForceCalculationTestF0", 1.3),
             ("VectorizationLennardJones", 35.0), ("VectorizationLennardJones1CLJ", 35.0),
             ("VectorizationCharge", 35.0), ("VectorizationChargeDipole", 35.0),
             ("VectorizationChargeQuadrupole", 35.0), ("VectorizationDipole", 35.0),
             ("VectorizationDipoleQuadrupole", 35.0), ("VectorizationQuadrupole", 35.0),
             ("VectorizationWater", 6.16), ("VectorizationMultiComponentMultiPotentials", 35.0)]
    for name, rc in cases:
        path = os.path.join(tin, name + ".inp")
        ps = psm.read_inp(path)
        res = run(["forces", path, rc, rc, 0])
        store("ref_" + name, ps, rc, rc, False, res)

    # (2) seeded periodic cases
    def case(name, ps, rc, rclj, steps=0, dt=0.0, keep=True, forces=True):
        path = os.path.join(tmp, name + ".inp")
        psm.write_inp(ps, path)
        ps = psm.read_inp(path)  # what the reference read, to the last bit
        if forces:
            res = run(["forces", path, rc, rclj, 1])
            store("per_" + name, ps, rc, rclj, True, res)
        if steps:
            res = run(["steps", path, rc, rclj, dt, steps])
            store("nve_" + name, ps, rc, rclj, True, res, dt, steps, keep)

    case("lj500", jitter(psm.lj_fcc(5, 0.8, 1.0, seed=11), 0.15, 12), 2.5, 2.5, steps=20, dt=0.002)
    case("lj864_rclj", jitter(psm.lj_fcc(6, 0.7, 1.2, seed=21, shifted=True, rc=2.2), 0.1, 22), 3.0, 2.2,
         steps=10, dt=0.002)
    mix = psm.mixture(500, 18.0, 300.0, seed=31)
    case("mix500", mix, 1.0, 1.0, steps=10, dt=9.118e-5)
    case("slab", psm.lj_slab(5, 0.73, 0.02, 0.9, seed=41), 2.5, 2.5, steps=10, dt=0.002)
    case("borders", psm.lj_on_cell_borders(11.0, 2.5, seed=51), 2.5, 2.5, steps=10, dt=0.002)
    case("lj4000j", jitter(psm.lj_fcc(10, 0.8, 1.0, seed=61), 0.1, 62), 2.5, 2.5)
    case("lj32000", psm.lj_fcc(20, 0.8, 1.0, seed=1), 2.5, 2.5, steps=100, dt=0.002, keep=False, forces=False)


if __name__ == "__main__":
    main()
