"""Region-wise temperature control (thermostats/TemperatureControl with
velocity-scaling regions) against the reference's own runs
(tests/golden/tc_*.npz, made by tests/golden/make_tempctl.py: NVE Leapfrog
with TemperatureControl::DoLoopsOverMolecules after each step's global
values).  1CLJ with two overlapping regions (3 slabs, x and z thermostated;
2 slabs, all directions, a temperature ramp), measuring every second step
between start and stop; the rotating 2CLJQ/1CLJD mixture with one region per
component (a ramp on the first, x and y on the second).

Tolerances: FP64 engine, per-step Upot/virial/kinetic sums to 5e-8 relative,
positions to 1e-9 of the box, velocities and angular momenta to 1e-7, and
the betas of the last measuring step per region and slab to 1e-7: the
engine sums in another order than the reference, and a thermostated run
carries those last-bit differences into every rescaling (the hot
quadrupolar mixture reaches 1.3e-8 in its kinetic sums over 10 steps).
"""
import json

import numpy as np
import pytest

import golden_io

NAMES = golden_io.names("tc_")


def test_golden_settings_are_consistent():
    for name in NAMES:
        ps, g = golden_io.load(name)
        tc = json.loads(str(g["tc_json"]))
        assert "<temperatureControl>" in str(g["tc_xml"])
        assert len(tc["regions"]) >= 2 and g["tcb"].shape[1] == 6
        # every region measured at least twice
        for r in range(len(tc["regions"])):
            assert len(set(g["tcb"][g["tcb"][:, 1] == r, 0])) >= 2


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_temperature_control_matches_reference(engine_mod, name):
    ps, g = golden_io.load(name)
    tc = json.loads(str(g["tc_json"]))
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64", skin=0.3)
    e.set_temperature_control(tc)
    e.forces()
    rec = e.run(float(g["dt"]), int(g["nsteps"]))
    steps = g["steps"][1:]
    for col, ref in ((0, steps[:, 1]), (1, steps[:, 2]), (2, steps[:, 3])):
        assert np.abs(rec[:, col] - ref).max() <= 5e-8 * np.abs(ref).max(), col
    tcb = g["tcb"]
    for r, reg in enumerate(tc["regions"]):
        rows = tcb[tcb[:, 1] == r]
        last = rows[rows[:, 0] == rows[:, 0].max()]
        bt, br = e.temperature_control_betas(r, reg["numslabs"])
        assert np.allclose(bt, last[:, 3], rtol=1e-7, atol=0), (r, bt - last[:, 3])
        assert np.allclose(br, last[:, 4], rtol=1e-7, atol=0), (r, br - last[:, 4])
    m = e.molecules()
    e.close()
    o = np.argsort(m["ids"])
    assert np.array_equal(m["ids"][o], g["out_ids"])
    assert np.abs(m["r"][o] - g["out_r"]).max() <= 1e-9 * np.abs(ps.box).max()
    assert np.abs(m["v"][o] - g["out_v"]).max() <= 1e-7 * np.abs(g["out_v"]).max()
    if np.abs(g["out_L"]).max() > 0:
        assert np.abs(m["L"][o] - g["out_L"]).max() <= 1e-7 * np.abs(g["out_L"]).max()


@pytest.mark.gpu
def test_temperature_control_step_by_step_equals_run(engine_mod):
    """md_integrate_pre / md_compute_forces / md_integrate_post with
    md_apply_temperature_control after each step equal md_run with the
    temperature control: the same kernels in the same order."""
    ps, g = golden_io.load("tc_lj500")
    tc = json.loads(str(g["tc_json"]))
    a = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64", skin=0.3)
    b = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64", skin=0.3)
    for e in (a, b):
        e.set_temperature_control(tc)
        e.forces()
    dt, n = float(g["dt"]), int(g["nsteps"])
    rows = []
    for k in range(1, n + 1):
        a.pre(dt)
        fo = a.forces()
        ko = a.post(dt)
        a.apply_temperature_control(k)
        rows.append([fo.upot, fo.virial, ko.summv2])
    rec = b.run(dt, n)
    ma, mb = a.molecules(), b.molecules()
    a.close()
    b.close()
    assert np.allclose(np.array(rows), rec[:, :3], rtol=1e-12, atol=0)
    assert np.array_equal(ma["v"], mb["v"]) and np.array_equal(ma["r"], mb["r"])
