"""The device velocity-scaling thermostat (md_set_thermostat / md_run and
md_apply_thermostat) against the reference's own NVT runs
(tests/golden/nvtt_*.npz, made by tests/golden/make_thermostat.py).

Tolerances: per-step Upot, virial, sum m v^2, sum I w^2 to 1e-8 relative and
final positions / velocities to 1e-7 (FP64; the device pow differs from the C
library's in the last bit); mixed precision to 1e-4 on the per-step sums."""
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


def _by_id(ids):
    return np.argsort(ids, kind="stable")


@pytest.mark.parametrize("name", golden_io.names("nvtt_"))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nvt_run_matches_reference(engine_mod, name, precision):
    ps, g = golden_io.load(name)
    skin = 0.3 * g["rc"] if precision == "mixed" else 0.0
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision=precision, skin=skin)
    e.set_thermostat(float(g["target_temperature"]))
    e.forces()
    rec = e.run(float(g["dt"]), int(g["nsteps"]))
    ref = g["steps"][1:, 1:]
    tol = 1e-8 if precision == "fp64" else 1e-4
    for col in range(4):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= tol * scale, col
    if precision == "fp64":
        m = e.molecules()
        a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
        for key, gk in (("r", "out_r"), ("v", "out_v"), ("L", "out_L")):
            assert np.abs(m[key][a] - g[gk][b]).max() <= 1e-7 * max(np.abs(g[gk]).max(), 1.0), key
    e.close()


def test_step_by_step_thermostat_equals_md_run(engine_mod):
    """md_integrate_pre / md_compute_forces / md_integrate_post /
    md_apply_thermostat (the drop-in's path) equal md_run with the thermostat,
    and the betas are those of the reference."""
    ps, g = golden_io.load("nvtt_lj500")
    T, dt = float(g["target_temperature"]), float(g["dt"])
    a = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64")
    a.set_thermostat(T)
    a.forces()
    ra = a.run(dt, 8)
    b = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64")
    b.set_thermostat(T)
    b.forces()
    betas = []
    for _ in range(8):
        b.pre(dt)
        b.forces()
        b.post(dt)
        betas.append(b.apply_thermostat())
    ma, mb = a.molecules(), b.molecules()
    assert np.abs(ma["v"] - mb["v"]).max() <= 1e-12 * np.abs(ma["v"]).max()
    assert np.allclose(np.array(betas), g["betas"][:8, 1:], rtol=1e-12, atol=0)
    assert ra.shape == (8, 4)
    a.close()
    b.close()


@pytest.mark.parametrize("name", golden_io.names("nvtc_"))
def test_componentwise_thermostats_match_reference(engine_mod, name):
    """Component c on thermostat c + 1 (tests/golden/nvtc_*.npz, the
    reference's several-thermostats path): per-step Upot and virial of md_run
    to 1e-8, final state to 1e-7; step by step, the betas of every thermostat
    to 1e-10 against the reference's."""
    ps, g = golden_io.load(name)
    dt, n = float(g["dt"]), int(g["nsteps"])
    targets = [float(x) for x in g["targets"]]
    ids = list(range(1, len(targets) + 1))
    a = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64")
    a.set_thermostats(ids, targets)
    a.forces()
    rec = a.run(dt, n)
    ref = g["steps"][1:, 1:]
    for col in range(2):  # the reference's kinetic columns hold the last thermostat's sums
        assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-8 * np.abs(ref[:, col]).max(), col
    m = a.molecules()
    a.close()
    i, j = _by_id(m["ids"]), _by_id(g["out_ids"])
    for key, gk in (("r", "out_r"), ("v", "out_v"), ("L", "out_L")):
        assert np.abs(m[key][i] - g[gk][j]).max() <= 1e-7 * max(np.abs(g[gk]).max(), 1.0), key
    b = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64")
    b.set_thermostats(ids, targets)
    b.forces()
    got = []
    for k in range(1, n + 1):
        b.pre(dt)
        b.forces()
        b.post(dt)
        b.apply_thermostat()
        for t in ids:
            got.append((k, t) + b.thermostat_betas(t))
    b.close()
    want = g["betas_c"]
    got = np.array(got)
    assert np.array_equal(got[:, :2], want[:, :2])
    assert np.allclose(got[:, 2:], want[:, 2:], rtol=1e-10, atol=0)
