"""Energy-drift reference: the reference implementation's own NVE run of the
1CLJ N=32,000 benchmark box (fcc 20^3 x 4, rho*=0.8, T*=1.0, rc=2.5,
dt=0.002) over 10,000 Leapfrog steps, built and driven as in make_golden.py.
Stores per-step Upot, virial, sum m v^2 (``drift_lj32000.npz``).

    python tests/golden/make_drift.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

STEPS = 10000


def main():
    ps = mg.psm.lj_fcc(20, 0.8, 1.0, seed=1)
    path = os.path.join(tempfile.mkdtemp(), "lj32000.inp")
    mg.psm.write_inp(ps, path)
    res = mg.run(["steps", path, 2.5, 2.5, 0.002, STEPS])
    steps = np.array(res["steps"])
    np.savez_compressed(os.path.join(HERE, "drift_lj32000.npz"), steps=steps, n=ps.n, dt=0.002, rc=2.5)
    e = steps[1:, 1] + 0.5 * steps[1:, 3]
    print("E0", e[0], "E_end", e[-1], "rel drift", (e[-1] - e[0]) / abs(e[0]))


if __name__ == "__main__":
    main()
