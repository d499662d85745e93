"""Energy drift over 10^4 NVE steps, against the reference's own run.

tests/golden/drift_lj32000.npz holds the reference implementation's Upot,
virial and sum m v^2 for every step of 10,000 Leapfrog steps of the
N=32,000 1CLJ box (fcc 20^3 x 4, rho*=0.8, T*=1.0, rc=2.5, truncated LJ,
dt=0.002), made by tests/golden/make_drift.py.  The total energy
E = Upot + sum m v^2 / 2 of a truncated potential jumps whenever a pair
crosses the cut-off, so E(t) first moves by the melting of the lattice and
then drifts slowly; both runs are chaotic, so they are compared statistically:

  * drift: |mean E over the last 1,000 steps - mean E over steps 100..1,100|,
    relative to |E(0)|, at most 1.1 x the reference's (10 % for the spread
    between chaotic trajectories);
  * the systematic change E(10^4) - E(0) within 5 % of the reference's;
  * the first 100 steps follow the reference's trajectory (FP64: Upot to
    1e-8 relative; mixed: 1e-6).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def _drift(E):
    return abs(E[-1000:].mean() - E[100:1100].mean()) / abs(E[0])


@pytest.mark.parametrize("precision,skin", [("fp64", 0.3), ("mixed", 0.3), ("mixed", 0.0)])
def test_energy_drift_no_worse_than_reference(engine_mod, precision, skin):
    from ls1gb300 import phasespace as psm
    d = np.load(os.path.join(HERE, "golden", "drift_lj32000.npz"))
    ref = d["steps"]
    E_ref = ref[1:, 1] + 0.5 * ref[1:, 3]
    ps = psm.lj_fcc(20, 0.8, 1.0, seed=1)
    e = engine_mod.Engine(ps, 2.5, 2.5, precision=precision, skin=skin)
    e.forces()
    rec = e.run(0.002, 10000)
    e.close()
    E = rec[:, 0] + 0.5 * rec[:, 2]
    assert np.all(np.isfinite(E))
    tol = 1e-8 if precision == "fp64" else 1e-6
    assert np.abs(rec[:100, 0] - ref[1:101, 1]).max() <= tol * np.abs(ref[1:101, 1]).max()
    assert _drift(E) <= 1.1 * _drift(E_ref), (_drift(E), _drift(E_ref))
    dE, dE_ref = E[-1] - E[0], E_ref[-1] - E_ref[0]
    assert abs(dE - dE_ref) <= 0.05 * abs(dE_ref), (dE, dE_ref)
