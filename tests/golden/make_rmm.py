"""Generate the reduced-memory-mode fixtures (rmm_*.npz) from the reference.

Runs the reference's own reduced memory mode (LeapfrogRMM, VCP1CLJRMM,
PositionCellProcessorRMM, VelocityCellProcessorRMM; the
-DENABLE_REDUCED_MEMORY_MODE build that ``oracle/ref/Makefile`` makes with
RMM=1 into ``oracle/_ref/``) through ``oracle/ref/ref_harness_rmm.cpp`` on
seeded periodic 1CLJ boxes written by ``ls1gb300.phasespace``: the initial
force pass with half the kick, then NVE steps.  Stores the inputs, the
per-step Upot, virial and sum of v^2, and the final positions and velocities.
Only this script reads the reference tree; the fixtures travel with the
repository.

    python tests/golden/make_rmm.py [--ref <ls1-mardyn tree>]   (default: oracle/refpath.py)
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
sys.path.insert(0, ROOT)
from ls1gb300 import phasespace as psm  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness_rmm_DPDP")


def run(args):
    p = subprocess.run([HARNESS] + [str(a) for a in args], capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"harness failed: {args}\n{p.stderr[-2000:]}")
    steps, mol = [], []
    for line in p.stdout.splitlines():
        t = line.split()
        if t and t[0] == "STEP":
            steps.append([float(x) for x in t[1:]])
        elif t and t[0] == "MOL":
            mol.append([float(x) for x in t[1:]])
    return np.array(steps), np.array(mol)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    a = ap.parse_args()
    if a.ref is None:
        from oracle.refpath import reference_tree
        a.ref = reference_tree()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={a.ref}", "RMM=1", "-j8"],
                   check=True)
    tmp = tempfile.mkdtemp()

    def case(name, ps, rc, dt, nsteps):
        path = os.path.join(tmp, name + ".inp")
        psm.write_inp(ps, path)
        steps, mol = run(["rmmsteps", path, rc, rc, dt, nsteps])
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            box=ps.box, components=json.dumps([dataclasses.asdict(c) for c in ps.components]),
                            mixing=np.array(ps.mixing).reshape(-1, 2), eps_rf=ps.eps_rf, ids=ps.ids, comp=ps.comp,
                            r=ps.r, v=ps.v, q=ps.q, L=ps.L, rc=rc, rc_lj=rc, periodic=1, dt=dt, nsteps=nsteps,
                            steps=steps, out_ids=mol[:, 0].astype(np.uint64), out_r=mol[:, 1:4], out_v=mol[:, 4:7])
        print(f"{name}: N={ps.n} out={mol.shape[0]} upot0={steps[0][1]} upot{nsteps}={steps[-1][1]}")

    def jittered(cells, rho, T, seed, mass=1.0):
        ps = psm.lj_fcc(cells, rho, T, seed=seed)
        ps.r = np.mod(ps.r + np.random.default_rng(seed + 1).uniform(-0.15, 0.15, ps.r.shape), ps.box)
        if mass != 1.0:
            ps.components = [psm.one_center_lj(m=mass)]
            ps.v = ps.v / np.sqrt(mass)
        return ps

    case("rmm_lj500", jittered(5, 0.8, 1.0, 11), 2.5, 0.002, 20)
    case("rmm_lj864_m17", jittered(6, 0.75, 0.9, 21, mass=1.7), 2.5, 0.003, 20)
    case("rmm_lj4000", jittered(10, 0.8, 1.0, 31), 2.5, 0.002, 30)


if __name__ == "__main__":
    main()
