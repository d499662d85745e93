"""Andersen regions of TemperatureControl (ControlRegionT::ControlTemperature,
thermostats/TemperatureControl.cpp:411-419).

The reference draws from one sequential generator (utils/Random.cpp) in the
container's traversal order, so its draws cannot be reproduced by a parallel
engine, nor from one thread count to the next under OpenMP.  The engine and
the oracle use the same counter-based draws instead (keyed by seed, step,
molecule id and region), so the engine is checked against the oracle
exactly: the same molecules selected, replaced v and L to 1e-13 of sqrt(T/m)
(log, sin and cos of CUDA and numpy differ in the last bits).  The
distribution itself, which is what the reference's runs share with these,
is checked on the oracle: the selected fraction is nu dt, the new v_d and
L_d are normal with variance T/m (L with the translational deviation, as the
reference's shared reserve deviate produces) and molecules outside the
region or not selected keep their state.
"""
import numpy as np
import pytest

from oracle.oracle import andersen_control


def _synthetic(n=200_000, seed=7):
    rng = np.random.default_rng(seed)
    ids = rng.permutation(np.arange(1, n + 1, dtype=np.uint64) * np.uint64(3))
    comp = rng.integers(0, 2, n).astype(np.int32)
    r = rng.uniform(0.0, 20.0, (n, 3))
    return ids, comp, r, rng.normal(size=(n, 3)), rng.normal(size=(n, 3))


REGION = dict(lower=[0.0, 0.0, 0.0], upper=[10.0, 20.0, 20.0], component=0)


def test_oracle_andersen_distribution():
    ids, comp, r, v, L = _synthetic()
    masses = [1.0, 2.5]
    T, nu_dt = 1.7, 0.25
    v2, L2, sel = andersen_control(ids, comp, r, v, L, masses, REGION, T, nu_dt, seed=11, step=40, index=0)
    inside = r[:, 0] < 10.0
    assert not sel[~inside].any()
    n_in = inside.sum()
    p = sel.sum() / n_in
    assert abs(p - nu_dt) < 5 * np.sqrt(nu_dt * (1 - nu_dt) / n_in)
    np.testing.assert_array_equal(v2[~sel], v[~sel])
    np.testing.assert_array_equal(L2[~sel], L[~sel])
    for c, m in enumerate(masses):
        s = sel & (comp == c)
        k = s.sum()
        for arr in (v2[s], L2[s]):
            z = arr / np.sqrt(T / m)
            assert np.abs(z.mean(0)).max() < 5 / np.sqrt(k)
            assert np.abs(z.var(0) - 1.0).max() < 5 * np.sqrt(2.0 / k)
        # v and L of a molecule come from independent draws
        assert abs(np.corrcoef(v2[s, 0], L2[s, 0])[0, 1]) < 5 / np.sqrt(k)


def test_oracle_andersen_keys():
    ids, comp, r, v, L = _synthetic(20_000)
    a = andersen_control(ids, comp, r, v, L, [1.0, 1.0], REGION, 1.0, 0.5, seed=3, step=8, index=0)
    b = andersen_control(ids, comp, r, v, L, [1.0, 1.0], REGION, 1.0, 0.5, seed=3, step=8, index=0)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    # order of the molecules does not matter
    o = np.argsort(ids)
    c = andersen_control(ids[o], comp[o], r[o], v[o], L[o], [1.0, 1.0], REGION, 1.0, 0.5, seed=3, step=8, index=0)
    np.testing.assert_array_equal(c[2], a[2][o])
    np.testing.assert_array_equal(c[0], a[0][o])
    # another step, seed or region index gives other selections
    for kw in (dict(seed=3, step=9, index=0), dict(seed=4, step=8, index=0), dict(seed=3, step=8, index=1)):
        d = andersen_control(ids, comp, r, v, L, [1.0, 1.0], REGION, 1.0, 0.5, **kw)
        inside = r[:, 0] < 10.0
        assert (d[2] != a[2])[inside].mean() > 0.3
    # component filter
    reg = dict(REGION, component=2)
    _, _, sel = andersen_control(ids, comp, r, v, L, [1.0, 1.0], reg, 1.0, 1.0, seed=3, step=8, index=0)
    np.testing.assert_array_equal(sel, (comp == 1) & (r[:, 0] < 10.0))


# ---------------------------------------------------------------- engine (GPU)
@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def _tc(regions, dt, seed=8624, start=0, freq=1, stop=10 ** 6):
    return dict(start=start, frequency=freq, stop=stop, regions=regions, timestep=dt, seed=seed)


def _andersen(lower, upper, T, nu, component=0):
    return dict(method="andersen", lower=lower, upper=upper, T=T, nu=nu, component=component)


def _masses(ps):
    return [c.mass_inertia()[0] for c in ps.components]


@pytest.mark.gpu
@pytest.mark.parametrize("system", ["lj", "mixture"])
def test_andersen_apply_matches_oracle(engine_mod, system):
    from ls1gb300 import phasespace as psm
    if system == "lj":
        ps = psm.lj_fcc(16, 0.8, 1.0, seed=4)
        rc, reg = 2.5, _andersen([0.0, 0.0, 0.0], [ps.box[0] / 2, None, None], 1.3, 40.0)
    else:
        ps = psm.mixture(2000, 18.0, 300.0, seed=2)
        rc, reg = 1.0, _andersen([0.0, 0.0, 0.0], [None, None, None], 300.0, 100.0, component=2)
    dt = 0.005
    e = engine_mod.Engine(ps, rc, precision="fp64")
    e.set_temperature_control(_tc([reg], dt, seed=99))
    before = e.molecules()
    e.apply_temperature_control(12)
    after = e.molecules()
    e.close()
    region = dict(lower=reg["lower"], upper=[ps.box[d] if u is None else u for d, u in enumerate(reg["upper"])],
                  component=reg["component"])
    v, L, sel = andersen_control(before["ids"], before["comp"], before["r"], before["v"], before["L"], _masses(ps),
                                 region, reg["T"], reg["nu"] * dt, seed=99, step=12, index=0)
    assert 0 < sel.sum() < len(sel)
    changed = np.any(after["v"] != before["v"], axis=1)
    np.testing.assert_array_equal(changed, sel)
    sd = np.sqrt(reg["T"] / np.asarray(_masses(ps))[before["comp"]])[:, None]
    assert np.abs((after["v"] - v) / sd).max() <= 1e-13
    assert np.abs((after["L"] - L) / sd).max() <= 1e-13
    np.testing.assert_array_equal(after["r"], before["r"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_andersen_inside_run(engine_mod, precision):
    """md_run with an Andersen region over the whole box that selects every
    molecule (nu dt = 1) beside a velocity-scaling region: after the last
    control step the velocities are the oracle's draws for that step at the
    final positions; a step that does not control leaves them alone."""
    from ls1gb300 import phasespace as psm
    ps = psm.lj_fcc(10, 0.8, 1.0, seed=6)
    dt, n = 0.004, 9
    vs = dict(lower=[0.0, 0.0, 0.0], upper=[None, None, None], T=1.0, component=0, numslabs=2, exponent=0.4,
              directions=7)
    reg = _andersen([0.0, 0.0, 0.0], [None, None, None], 2.0, 1.0 / dt)
    e = engine_mod.Engine(ps, 2.5, precision=precision, skin=0.3)
    e.set_temperature_control(_tc([vs, reg], dt, seed=5, freq=3))
    e.forces()
    e.run(dt, n)
    m = e.molecules()
    e.run(dt, 1)  # step 10: no control
    m2 = e.molecules()
    e.close()
    region = dict(lower=[0.0] * 3, upper=list(ps.box), component=0)
    v, L, sel = andersen_control(m["ids"], m["comp"], m["r"], m["v"] * 0, m["L"] * 0, [1.0], region, 2.0, 1.0,
                                 seed=5, step=n, index=1)
    assert sel.all()
    assert np.abs(m["v"] - v).max() <= 1e-13 * np.sqrt(2.0)
    assert abs((m["v"] ** 2).sum() / (3 * ps.n) - 2.0) < 5 * np.sqrt(2.0 / (3 * ps.n)) * 2.0
    assert np.any(m2["v"] != m["v"])  # the step itself moves them
    assert np.abs(m2["v"] - m["v"]).max() < 0.5


@pytest.mark.gpu
def test_andersen_rejects_invalid(engine_mod):
    from ls1gb300 import phasespace as psm
    ps = psm.lj_fcc(5, 0.8, 1.0, seed=1)
    e = engine_mod.Engine(ps, 2.5, precision="fp64")
    reg = _andersen([0.0] * 3, [None] * 3, 1.0, 10.0)
    with pytest.raises(engine_mod.EngineError):
        e.set_temperature_control(_tc([reg], 0.0))
    with pytest.raises(engine_mod.EngineError):
        e.set_temperature_control(_tc([dict(reg, nu=-1.0)], 0.01))
    e.close()
