"""Reduced memory mode (the reference's ENABLE_REDUCED_MEMORY_MODE build:
LeapfrogRMM + VCP1CLJRMM + PositionCellProcessorRMM +
VelocityCellProcessorRMM).

Pinned against the reference's own reduced-memory-mode runs
(tests/golden/rmm_*.npz, written by tests/golden/make_rmm.py from the
reference built with -DENABLE_REDUCED_MEMORY_MODE): the oracle's restatement
to 1e-12 (records) and 1e-12 / 1e-11 (final positions / velocities), the
engine in FP64 to 1e-9 and in mixed precision to the NVE tolerances of the
other parity tests.  The oracle's reduced mode is also the oracle's Leapfrog
with half-step velocities: both are the same Stoermer-Verlet scheme, so the
positions, Upot and virial of every step agree to rounding, and the reduced
mode's velocities are the Leapfrog velocities plus a half kick dt/(2m) F.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle


def _lj_box(cells=6, rho=0.8, T=1.0, seed=3, mass=1.0):
    """fcc lattice with seeded displacements of up to 0.1 sigma (on the
    perfect lattice every force vanishes)."""
    from ls1gb300 import phasespace as psm
    ps = psm.lj_fcc(cells, rho, T, seed=seed)
    rng = np.random.default_rng(seed + 100)
    ps.r = np.mod(ps.r + rng.uniform(-0.1, 0.1, ps.r.shape), ps.box)
    if mass != 1.0:
        c = ps.components[0]
        ps.components = [psm.one_center_lj(m=mass)]
        assert c.lj[0].eps == 1.0
        ps.v = ps.v / np.sqrt(mass)
    return ps


def _golden(name):
    import golden_io as G
    ps, g = G.load(name)
    return ps, g, ps.components[0].mass_inertia()[0]


RMM_GOLDEN = ["rmm_lj500", "rmm_lj864_m17", "rmm_lj4000"]


def _by_id(m):
    o = np.argsort(m["ids"])
    return {k: (v[o] if hasattr(v, "shape") and v.shape[:1] == o.shape else v) for k, v in m.items()}


# ---------------------------------------------------------------- oracle (CPU)
@pytest.mark.parametrize("mass", [1.0, 1.7])
def test_oracle_rmm_is_leapfrog_with_half_step_velocities(mass):
    ps = _lj_box(mass=mass)
    dt, n = 0.002, 20
    lf = Oracle(ps, 2.5, threads=2)
    lf.rebin()
    lf.forces()
    rec_lf = lf.run(dt, n)
    rm = Oracle(ps, 2.5, threads=2)
    fo = rm.rmm_forces(0.5 * dt / mass)  # Simulation::prepare_start halves dt/m
    rec_rm = rm.rmm_run(dt, n)
    a, b = _by_id(lf.molecules()), _by_id(rm.molecules())
    assert np.abs(a["r"] - b["r"]).max() <= 1e-12
    for col in (0, 1):
        assert np.abs(rec_lf[:, col] - rec_rm[:, col]).max() <= 1e-12 * np.abs(rec_lf[:, col]).max()
    # v(n + 1/2) = v(n) + dt/(2m) F(n)
    assert np.allclose(b["v"], a["v"] + 0.5 * dt / mass * a["F"], rtol=0, atol=1e-12)
    # the velocity sums carry no mass (VelocityCellProcessorRMM)
    assert np.isclose(rec_rm[-1, 2], (b["v"] ** 2).sum(), rtol=1e-13)
    assert np.all(rec_rm[:, 3] == 0.0)
    assert fo.site_pairs[0] > 0


@pytest.mark.parametrize("name", RMM_GOLDEN)
def test_oracle_rmm_matches_the_reference_rmm_run(name):
    """The initial force pass with half the kick, then NVE steps, against the
    reference's own reduced-memory-mode run of the same input."""
    ps, g, m = _golden(name)
    dt, n = float(g["dt"]), int(g["nsteps"])
    o = Oracle(ps, g["rc"], threads=4)
    fo = o.rmm_forces(0.5 * dt / m)
    rec = o.rmm_run(dt, n)
    st = g["steps"]
    assert abs(fo.upot - st[0, 1]) <= 1e-12 * abs(st[0, 1])
    assert abs(fo.virial - st[0, 2]) <= 1e-12 * abs(st[0, 2])
    for col in range(3):  # Upot, virial, sum v^2 of every step
        assert np.abs(rec[:, col] - st[1:, col + 1]).max() <= 1e-12 * np.abs(st[1:, col + 1]).max(), col
    mo = _by_id(o.molecules())
    np.testing.assert_array_equal(mo["ids"], g["out_ids"])
    assert np.abs(mo["r"] - g["out_r"]).max() <= 1e-12
    assert np.abs(mo["v"] - g["out_v"]).max() <= 1e-11


def test_oracle_rmm_velocity_pass():
    ps = _lj_box(mass=2.5)
    o = Oracle(ps, 2.5, threads=2)
    ko = o.rmm_velocities()
    assert ko.n == ps.n and ko.rot_dof == 0 and ko.sumIw2 == 0.0
    assert np.isclose(ko.summv2, (ps.v ** 2).sum(), rtol=1e-13)


# ---------------------------------------------------------------- engine (GPU)
@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rmm_force_pass_matches_oracle(engine_mod, precision):
    ps = _lj_box(cells=8, mass=1.3)
    k = 0.001 / 1.3
    o = Oracle(ps, 2.5, threads=4)
    fo_ref = o.rmm_forces(k)
    ref = _by_id(o.molecules())
    e = engine_mod.Engine(ps, 2.5, precision=precision, skin=0.3)
    fo = e.rmm_forces(k)
    got = _by_id(e.molecules())
    e.close()
    assert int(fo.site_pairs[0]) == int(fo_ref.site_pairs[0])
    dv_ref = ref["v"] - ps.v[np.argsort(ps.ids)]
    dv = got["v"] - ps.v[np.argsort(ps.ids)]
    if precision == "fp64":
        assert np.abs(dv - dv_ref).max() <= 1e-10 * np.abs(dv_ref).max()
        assert abs(fo.upot - fo_ref.upot) <= 1e-10 * abs(fo_ref.upot)
        assert abs(fo.virial - fo_ref.virial) <= 1e-10 * abs(fo_ref.virial)
    else:
        # the kick is k F with F the FP32 force: relative rms 1e-5 of the force error
        rms = np.sqrt(((dv - dv_ref) ** 2).sum(1).mean() / (dv_ref ** 2).sum(1).mean())
        assert rms <= 1e-5
        assert abs(fo.upot - fo_ref.upot) <= 1e-5 * abs(fo_ref.upot)
    np.testing.assert_array_equal(got["r"], ps.r[np.argsort(ps.ids)])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rmm_run_matches_oracle(engine_mod, precision):
    """30 LeapfrogRMM steps from the initial half-kick force pass; the list
    skin makes some steps rebuild and others reuse the list."""
    ps = _lj_box(cells=8, mass=1.3)
    dt, n = 0.002, 30
    o = Oracle(ps, 2.5, threads=4)
    o.rmm_forces(0.5 * dt / 1.3)
    ref = o.rmm_run(dt, n)
    e = engine_mod.Engine(ps, 2.5, precision=precision, skin=0.15)
    e.rmm_forces(0.5 * dt / 1.3)
    rec = e.rmm_run(dt, n)
    m = _by_id(e.molecules())
    e.close()
    mo = _by_id(o.molecules())
    if precision == "fp64":
        for col in range(3):
            assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-9 * np.abs(ref[:, col]).max(), col
        assert np.abs(m["r"] - mo["r"]).max() <= 1e-10
        assert np.abs(m["v"] - mo["v"]).max() <= 1e-9
    else:
        for col in range(3):
            assert np.abs(rec[:, col] - ref[:, col]).max() <= 2e-5 * np.abs(ref[:, col]).max(), col
        assert np.abs(m["r"] - mo["r"]).max() <= 1e-6
    assert np.all(rec[:, 3] == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", RMM_GOLDEN)
def test_rmm_run_matches_the_reference_rmm_run(engine_mod, name, precision):
    """md_rmm_forces (half kick) + md_rmm_run against the reference's own
    reduced-memory-mode run: FP64 1e-9; mixed precision 2e-5 on the records
    and 1e-6 on the final positions, as the other NVE parity tests."""
    ps, g, m = _golden(name)
    dt, n = float(g["dt"]), int(g["nsteps"])
    e = engine_mod.Engine(ps, g["rc"], precision=precision, skin=0.2)
    fo = e.rmm_forces(0.5 * dt / m)
    rec = e.rmm_run(dt, n)
    got = _by_id(e.molecules())
    e.close()
    st = g["steps"]
    tol = 1e-9 if precision == "fp64" else 2e-5
    assert abs(fo.upot - st[0, 1]) <= tol * abs(st[0, 1])
    for col in range(3):
        assert np.abs(rec[:, col] - st[1:, col + 1]).max() <= tol * np.abs(st[1:, col + 1]).max(), col
    np.testing.assert_array_equal(got["ids"], g["out_ids"])
    if precision == "fp64":
        assert np.abs(got["r"] - g["out_r"]).max() <= 1e-10
        assert np.abs(got["v"] - g["out_v"]).max() <= 1e-9
    else:
        assert np.abs(got["r"] - g["out_r"]).max() <= 1e-6


@pytest.mark.gpu
def test_rmm_calls_equal_run(engine_mod):
    """Positions, forces with dt/m and velocity sums called one by one give
    the same FP64 state and records as md_rmm_run (same kernels, same
    per-warp sums)."""
    ps = _lj_box(cells=7, mass=1.0)
    dt, n = 0.002, 12
    a = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.2)
    b = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.2)
    ra = engine_mod.GpuLinkedCells.__new__(engine_mod.GpuLinkedCells)
    ra.engine, ra._cutoff = a, 2.5
    integ = engine_mod.GpuLeapfrogRMM(dt, 1.0)
    integ.prepare(ra)
    rows = []
    for _ in range(n):
        integ.eventNewTimestep(ra)
        fo = integ.traverseCells(ra)
        ko = integ.eventForcesCalculated(ra)
        rows.append([fo.upot, fo.virial, ko.summv2, ko.sumIw2])
    b.rmm_forces(0.5 * dt)
    rec = b.rmm_run(dt, n)
    ma, mb = a.molecules(), b.molecules()
    a.close()
    b.close()
    np.testing.assert_array_equal(np.array(rows), rec)
    for k in ("ids", "r", "v"):
        np.testing.assert_array_equal(ma[k], mb[k])


@pytest.mark.gpu
def test_rmm_mixed_fused_drift_equals_calls(engine_mod):
    """Mixed precision: md_rmm_run puts the next step's drift into the pair
    kernel (two position buffers).  60 steps (two graph chunks and an eager
    remainder, several rebuilds) against the drift / force / velocity calls:
    positions, velocities, Upot and virial bit for bit; the velocity sums are
    FP32 products in the fused kernel (1e-6)."""
    ps = _lj_box(cells=7, mass=1.0)
    ps.v = ps.v * 1.5
    dt, n = 0.004, 60
    a = engine_mod.Engine(ps, 2.5, precision="mixed", skin=0.2)
    b = engine_mod.Engine(ps, 2.5, precision="mixed", skin=0.2)
    ra = engine_mod.GpuLinkedCells.__new__(engine_mod.GpuLinkedCells)
    ra.engine, ra._cutoff = a, 2.5
    integ = engine_mod.GpuLeapfrogRMM(dt, 1.0)
    integ.prepare(ra)
    rows = []
    for _ in range(n):
        integ.eventNewTimestep(ra)
        fo = integ.traverseCells(ra)
        ko = integ.eventForcesCalculated(ra)
        rows.append([fo.upot, fo.virial, ko.summv2])
    rows = np.array(rows)
    b.rmm_forces(0.5 * dt)
    rec = b.rmm_run(dt, n)
    assert b.rebuilds() >= 3
    ma, mb = a.molecules(), b.molecules()
    a.close()
    b.close()
    np.testing.assert_array_equal(rec[:, :2], rows[:, :2])
    assert np.abs(rec[:, 2] - rows[:, 2]).max() <= 1e-6 * np.abs(rows[:, 2]).max()
    for k in ("ids", "r", "v"):
        np.testing.assert_array_equal(ma[k], mb[k])


@pytest.mark.gpu
def test_rmm_positions_follow_leapfrog_at_scale(engine_mod):
    """108,000 molecules, 40 steps: the reduced mode's positions, Upot and
    virial are the Leapfrog ones (FP64, same list schedule up to rounding)."""
    ps = _lj_box(cells=30, seed=5)
    dt, n = 0.002, 40
    lf = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.3)
    lf.forces()
    rec_lf = lf.run(dt, n)
    rm = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.3)
    rm.rmm_forces(0.5 * dt)
    rec_rm = rm.rmm_run(dt, n)
    a, b = _by_id(lf.molecules()), _by_id(rm.molecules())
    lf.close()
    rm.close()
    assert np.abs(a["r"] - b["r"]).max() <= 1e-10
    for col in (0, 1):
        assert np.abs(rec_lf[:, col] - rec_rm[:, col]).max() <= 1e-11 * np.abs(rec_lf[:, col]).max(), col
    assert np.allclose(b["v"], a["v"] + 0.5 * dt * a["F"], rtol=0, atol=1e-10)


@pytest.mark.gpu
def test_rmm_rejects_other_systems(engine_mod):
    from ls1gb300 import phasespace as psm
    ps = psm.mixture(500, 18.0, 300.0, seed=1)
    e = engine_mod.Engine(ps, 1.0, precision="fp64")
    with pytest.raises(engine_mod.EngineError):
        e.rmm_forces(1e-3)
    e.close()
    ps1 = _lj_box(cells=5)
    e = engine_mod.Engine(ps1, 2.5, precision="fp64")
    with pytest.raises(engine_mod.EngineError):  # no initial force pass yet
        e.rmm_run(0.002, 3)
    e.close()
