"""ResultWriter output (io/ResultWriter.cpp) and the global values behind
it (Domain::calculateGlobalValues, Domain::getGlobalPressure) against
`.res` files the reference's own ResultWriter wrote (tests/golden/res_*.npz,
made by tests/golden/make_results.py): NVE and NVT 1CLJ runs and an NVT run
of the rotating 2CLJQ/1CLJD mixture, every step written, sliding averages
over 7 steps (so the windows wrap).

The oracle's records give the same lines to the 11 printed digits (1e-9
relative allowed for rounding of the last digit); the engine's FP64 records
to 1e-8.  The layout (column widths, header) is compared as text.
"""
import numpy as np
import pytest

import golden_io
from ls1gb300 import results as R
from oracle.oracle import Oracle

NAMES = golden_io.names("res_")


def _golden(name):
    ps, g = golden_io.load(name)
    return ps, g, str(g["res_lines"]).splitlines()


def _write(tmp_path, name, rec, ps, g):
    n, rot, box = R.system_constants(ps)
    T = float(g["target_temperature"])
    rw = R.write_results(str(tmp_path / name), rec, n, rot, box, float(g["dt"]),
                         target_temperature=T if T > 0 else None, write_frequency=int(g["write_frequency"]),
                         accumulation_steps=int(g["accumulation_steps"]), write_precision=int(g["write_precision"]))
    rw.finish()
    lines = open(rw.path).read().splitlines()
    assert lines[0].startswith("# ls1 MarDyn simulation started at ")
    assert lines[-1].startswith("# ls1 mardyn simulation finished at ")
    return lines[1:-1]


def _compare(ours, gold, rtol):
    assert len(ours) == len(gold)
    assert ours[:2] == gold[:2]  # averaging comment and column header, as text
    for a, b in zip(ours[2:], gold[2:]):
        assert len(a) == len(b)
        fa, fb = a.split(), b.split()
        assert fa[0] == fb[0] and fa[-1] == fb[-1]  # step, N
        x, y = np.array(fa[1:-1], float), np.array(fb[1:-1], float)
        assert np.all(np.abs(x - y) <= rtol * np.maximum(np.abs(y), 1e-300)), (a, b)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_records_give_reference_results(name, tmp_path):
    ps, g, gold = _golden(name)
    o = Oracle(ps, g["rc"], g["rc_lj"], threads=4)
    o.rebin()
    o.forces()
    T = float(g["target_temperature"])
    if T > 0:
        o.set_thermostat(T)
    rec = o.run(float(g["dt"]), int(g["nsteps"]))
    _compare(_write(tmp_path, name, rec, ps, g), gold, 1e-9)


def test_global_values_formulas():
    """Domain::calculateGlobalValues / getGlobalPressure on one record."""
    g = R.global_values([-10.0, 30.0, 12.0, 3.0], 4, 6, [2.0, 2.0, 5.0], target_temperature=1.5, upot_corr=-1.0,
                        virial_corr=2.0)
    T = (12.0 + 3.0) / (3 * 4 + 6)
    rho = 4 / 20.0
    assert g.upot == -11.0 and g.virial == 32.0 and g.temperature == T
    assert g.pressure == T * rho + rho * (32.0 / 4) / 3.0
    assert g.ukin == 7.5
    assert g.beta_trans == (3.0 * 4 * 1.5 / 12.0) ** 0.4 and g.beta_rot == (6 * 1.5 / 3.0) ** 0.4
    nve = R.global_values([-10.0, 30.0, 12.0, 3.0], 4, 0, [2.0, 2.0, 5.0])
    assert nve.beta_trans == nve.beta_rot == 1.0 and nve.ukin == 6.0  # no rotation: sum I w^2 ignored


def test_accumulator_window_wraps():
    a = R.Accumulator(3)
    for v in (1.0, 2.0, 4.0, 8.0):
        a.add(v)
    assert a.size == 3 and a.average() == (8.0 + 2.0 + 4.0) / 3  # storage order after the wrap


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_engine_records_give_reference_results(engine_mod, name, tmp_path):
    ps, g, gold = _golden(name)
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64", skin=0.3)
    T = float(g["target_temperature"])
    if T > 0:
        e.set_thermostat(T)
    e.forces()
    rec = e.run(float(g["dt"]), int(g["nsteps"]))
    e.close()
    _compare(_write(tmp_path, name, rec, ps, g), gold, 1e-8)
