"""The planar long-range correction (md_planar_init / md_planar_apply)
against the reference's own runs (tests/golden/planar_*.npz, made by
tests/golden/make_planar.py): NVE steps with Planar::calculateLongRange
between the traversal and calcFM, slabs along y, profiles every
`frequency` calls, force corrections in a y region.

Tolerances (FP64): the per-call UpotCorr and VirialCorr to 1e-10 relative
(the reference sums them over molecules in an OpenMP reduction, so its
last bits depend on the thread count); per-step Upot, virial and sum m v^2
to 1e-8 relative and final positions, velocities, forces and virials to
1e-7 of their largest magnitude, the bounds of the NVE parity tests (the
rotational update of the mixture rounds differently in the last bits and
the difference grows over the steps).  Mixed precision (single-centre
slab): corrections to 1e-6 relative."""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def _run(engine_mod, name, precision):
    ps, g = golden_io.load(name)
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision=precision, skin=0.0 if precision == "fp64" else 0.3)
    e.planar_init(int(g["slabs"]), int(g["frequency"]), region=tuple(g["region"]),
                  target_temperature=float(g["target_temperature"]))
    dt, n = float(g["dt"]), int(g["nsteps"])
    f = e.forces()
    lrc = [e.planar_apply()]
    steps = [(f.upot, f.virial, np.nan, np.nan)]
    for _ in range(n):
        e.pre(dt)
        f = e.forces()
        lrc.append(e.planar_apply())
        k = e.post(dt)
        steps.append((f.upot, f.virial, k.summv2, k.sumIw2))
    m = e.molecules()
    e.close()
    return g, np.array(lrc), np.array(steps), m


@pytest.mark.parametrize("name", golden_io.names("planar_"))
def test_planar_run_matches_reference(engine_mod, name):
    g, lrc, steps, m = _run(engine_mod, name, "fp64")
    ref = g["lrc"]
    assert lrc.shape == ref.shape
    for col in range(2):
        assert np.abs(lrc[:, col] - ref[:, col]).max() <= 1e-10 * np.abs(ref[:, col]).max(), (col, lrc, ref)
    rs = g["steps"]
    for col in (1, 2):
        assert np.abs(steps[:, col - 1] - rs[:, col]).max() <= 1e-8 * np.abs(rs[:, col]).max(), col
    assert np.abs(steps[1:, 2] - rs[1:, 3]).max() <= 1e-8 * np.abs(rs[1:, 3]).max()
    o = np.argsort(m["ids"])
    assert np.array_equal(m["ids"][o], g["out_ids"])
    for k, f in (("r", "out_r"), ("v", "out_v"), ("F", "F"), ("Vi", "Vi")):
        assert np.abs(m[k][o] - g[f]).max() <= 1e-7 * max(np.abs(g[f]).max(), 1e-300), k


def test_planar_mixed_precision(engine_mod):
    g, lrc, steps, m = _run(engine_mod, "planar_slab1clj", "mixed")
    ref = g["lrc"]
    for col in range(2):
        assert np.abs(lrc[:, col] - ref[:, col]).max() <= 1e-6 * np.abs(ref[:, col]).max(), col


def test_planar_force_region(engine_mod):
    """Outside the force region only the virial changes: with the region set
    to an empty y range the forces equal those without the correction."""
    from ls1gb300 import phasespace as psm
    ps, g = golden_io.load("planar_slab1clj")
    a = engine_mod.Engine(ps, g["rc"], precision="fp64")
    a.forces()
    F0 = a.molecules()["F"]
    a.planar_init(100, 1, region=(-2.0, -1.0))
    u, w = a.planar_apply()
    m = a.molecules()
    a.close()
    assert np.array_equal(m["F"], F0)
    assert u < 0 and w < 0
