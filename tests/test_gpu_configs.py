"""Precision and parity at the benchmark configurations' full sizes.

  * C2a: 1CLJ fcc 100^3 x 4 = 4,000,000 molecules, rho*=0.75, T*=0.9, rc=3.0;
  * C2b: the vapour-liquid slab, 3,200,000 molecules (liquid rho*=0.73 in the
    middle third of a box elongated 3x in z, vapour rho*=0.02), rc=3.0;
  * C3: the 2CLJQ/1CLJD mixture, 1,000,188 molecules, n=18 nm^-3, T=300 K,
    rc=1 nm, reaction field eps_RF=1e10.

Each state is taken after a short mixed-precision NVE run from the seeded
generator (the lattice has begun to melt), then evaluated by the mixed and
the FP64 kernels and by the oracle (OpenMP C08, all host cores).  Bars:

  * interacting molecule and site pair counts: mixed == FP64 == oracle, exact;
  * FP64 kernel vs oracle: forces to 1e-10 relative to the largest force;
    Upot and virial to 1e-10 relative;
  * mixed vs FP64: relative rms force error <= 1e-5 (the stated target),
    torques <= 1e-4 (multi-site, as on the golden cases), Upot, virial and
    pressure <= 1e-6 relative for single-centre LJ and <= 1e-5 for the
    multipolar mixture (whose virial is a sum of large cancelling site-pair
    terms; measured 1.7e-6 on a GB300).

And the drift bar at the C2a state point on a 1,000,188-molecule subset
(fcc 63^3 x 4): 10^4 NVE steps in each precision from the same start; the
mixed run's drift (|mean E over the last 1,000 steps - mean E over steps
100..1,100| / |E0|) is at most 1.1x the FP64 run's plus 1e-6 (FP64 itself is
pinned against the reference's own 10^4-step run at N=32,000 in
test_gpu_drift.py).
"""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def mods():
    import importlib
    import build as eb
    eb.build()
    return (importlib.import_module("ls1gb300.engine"), importlib.import_module("ls1gb300.phasespace"),
            importlib.import_module("ls1gb300.precision"))


CONFIGS = {
    "C2a_lj4m": (lambda psm: psm.lj_fcc(100, 0.75, 0.9, seed=2024), 3.0, 0.002, 0.25, 30),
    "C2b_slab3m": (lambda psm: psm.lj_slab(91, 0.73, 0.02, 0.9, seed=2025), 3.0, 0.002, 0.25, 30),
    "C3_mix1m": (lambda psm: psm.mixture(1_000_000, 18.0, 300.0, seed=2026), 1.0, 9.118e-5, 0.1, 20),
}


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_precision_and_pair_counts_at_full_size(mods, name):
    E, psm, P = mods
    gen, rc, dt, skin, nsteps = CONFIGS[name]
    ps0 = gen(psm)
    e = E.Engine(ps0, rc, precision="mixed", skin=skin)
    e.forces()
    e.run(dt, nsteps, record=False)
    ps = P.state_of(e.molecules(), ps0)
    fom = e.forces()
    mm = e.molecules()
    e.close()
    rep = P.report(ps, rc, skin=skin, mixed_forces=(fom, mm))
    print(name, rep)
    assert rep["pairs_equal"], rep
    assert rep["force_rel_rms"] <= 1e-5, rep
    if "torque_rel_rms" in rep:
        assert rep["torque_rel_rms"] <= 1e-4, rep
    tol = 1e-5 if "torque_rel_rms" in rep else 1e-6
    for k in ("upot_rel", "virial_rel", "pressure_rel"):
        assert rep[k] <= tol, rep
    # FP64 kernel and pair counts against the oracle on the same state
    e6 = E.Engine(ps, rc, precision="fp64", skin=0.0)
    fo6 = e6.forces()
    m6 = e6.molecules()
    e6.close()
    o = Oracle(ps, rc, threads=THREADS)
    o.rebin()
    foo, _ = o.forces()
    mo = o.molecules()
    assert fo6.mol_pairs == foo.mol_pairs and fom.mol_pairs == foo.mol_pairs
    assert list(fo6.site_pairs) == list(foo.site_pairs) and list(fom.site_pairs) == list(foo.site_pairs)
    i6, io = np.argsort(m6["ids"], kind="stable"), np.argsort(mo["ids"], kind="stable")
    F6, Fo = m6["F"][i6], mo["F"][io]
    assert np.abs(F6 - Fo).max() <= 1e-10 * np.abs(Fo).max()
    assert abs(fo6.upot - foo.upot) <= 1e-10 * abs(foo.upot)
    assert abs(fo6.virial - foo.virial) <= 1e-10 * abs(foo.virial)


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_newton3_at_full_size(mods, name):
    """The Newton-3 paths at the benchmark sizes -- cluster pairs for the
    1CLJ configurations, the multi-site kernels' half rows with atomics for
    the mixture: the same interacting pair counts as the FP64 kernel
    (exact), relative rms force error <= 1e-5 and Upot, virial, pressure
    <= 1e-6 against it (mixture: torques <= 1e-4, sums <= 1e-5, the bars of
    the rows above)."""
    E, psm, P = mods
    gen, rc, dt, skin, nsteps = CONFIGS[name]
    ps0 = gen(psm)
    e = E.Engine(ps0, rc, precision="mixed", skin=skin, pair_scheme="newton3")
    e.forces()
    e.run(dt, nsteps, record=False)
    assert e.time_kernels(1).pair_scheme == 1
    ps = P.state_of(e.molecules(), ps0)
    fom = e.forces()
    mm = e.molecules()
    e.close()
    rep = P.report(ps, rc, skin=skin, mixed_forces=(fom, mm))
    print(name, "newton3", rep)
    assert rep["pairs_equal"], rep
    assert rep["force_rel_rms"] <= 1e-5, rep
    if "torque_rel_rms" in rep:
        assert rep["torque_rel_rms"] <= 1e-4, rep
    tol = 1e-5 if "torque_rel_rms" in rep else 1e-6
    for k in ("upot_rel", "virial_rel", "pressure_rel"):
        assert rep[k] <= tol, rep


def _drift(En):
    return abs(En[-1000:].mean() - En[100:1100].mean()) / abs(En[0])


def test_mixed_drift_no_worse_than_fp64_at_the_c2a_state_point(mods):
    E, psm, _ = mods
    ps = psm.lj_fcc(63, 0.75, 0.9, seed=2024)
    drift = {}
    for prec in ("fp64", "mixed"):
        e = E.Engine(ps, 3.0, precision=prec, skin=0.25)
        e.forces()
        rec = e.run(0.002, 10000)
        e.close()
        En = rec[:, 0] + 0.5 * rec[:, 2]
        assert np.all(np.isfinite(En))
        drift[prec] = _drift(En)
    print("drift", drift)
    assert drift["mixed"] <= 1.1 * drift["fp64"] + 1e-6, drift
