"""Pin the C oracle against the reference's own outputs (tests/golden/*.npz).

The golden vectors were produced by the reference implementation itself
(built from its sources by oracle/ref/Makefile, driven by
oracle/ref/ref_harness.cpp; see tests/golden/make_golden.py).  The oracle
restates the reference's arithmetic operation by operation, so it must agree
to rounding of the summation order:
  * cell assignment, kernel-call and macroscopic pair counts: exact
  * per-molecule F, M, Vi and Upot/virial: 1e-12 relative to the largest
    magnitude in the case (the reference's own DPDP tolerance between its two
    kernels, VectorizedCellProcessorTest.cpp:143-147, 229-233)
  * NVE trajectories (Leapfrog, periodic halo): per-step sums 1e-10 relative,
    final state 1e-9 absolute.
"""
import numpy as np
import pytest

import golden_io
from oracle.oracle import Oracle

FORCE_CASES = golden_io.names("ref_") + golden_io.names("per_")
NVE_CASES = golden_io.names("nve_")


def _by_id(ids):
    return np.argsort(ids, kind="stable")


def _rel(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


@pytest.mark.parametrize("name", FORCE_CASES)
def test_oracle_forces_match_reference(name):
    ps, g = golden_io.load(name)
    o = Oracle(ps, g["rc"], g["rc_lj"], (1, 1, 1) if g["periodic"] else (0, 0, 0), threads=4)
    st = o.rebin()
    assert list(st.cells) == list(g["grid"])
    fo, kernel = o.forces()
    m = o.molecules()
    a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
    assert np.array_equal(m["ids"][a], g["out_ids"][b])
    assert np.array_equal(o.cells()[a], g["out_cell"][b])
    for key in ("F", "M", "Vi"):
        if np.abs(g[key]).max() > 0:
            assert _rel(m[key][a], g[key][b]) < 1e-12, key
    assert abs(fo.upot - float(g["upot"])) <= 1e-12 * max(1.0, abs(float(g["upot"])))
    assert abs(fo.virial - float(g["virial"])) <= 1e-12 * max(1.0, abs(float(g["virial"])))
    counts = g["counts"]
    assert kernel[0] == counts[0]                      # molecule distance checks
    assert list(kernel[1:].astype(np.int64)) == list(counts[1::2].astype(np.int64))
    assert list(fo.site_pairs) == list(counts[2::2].astype(np.int64))


@pytest.mark.parametrize("name", NVE_CASES)
def test_oracle_nve_matches_reference(name):
    ps, g = golden_io.load(name)
    o = Oracle(ps, g["rc"], g["rc_lj"], (1, 1, 1), threads=8)
    o.rebin()
    fo, _ = o.forces()
    steps = g["steps"]
    assert abs(fo.upot - steps[0][1]) <= 1e-10 * abs(steps[0][1])
    rec = o.run(float(g["dt"]), int(g["nsteps"]))
    ref = steps[1:, 1:]
    for col in range(4):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-10 * scale, col
    m = o.molecules()
    if "out_r" in g:
        a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
        for key, gk in (("r", "out_r"), ("v", "out_v"), ("q", "out_q"), ("L", "out_L")):
            assert np.abs(m[key][a] - g[gk][b]).max() < 1e-9, key
    else:
        assert np.allclose(m["r"].sum(axis=0), g["out_r_sum"], rtol=1e-12)


def test_known_answers_u0_f0():
    """Analytic known answers of VectorizedCellProcessorTest.cpp:45-134."""
    ps, g = golden_io.load("ref_ForceCalculationTestU0")
    o = Oracle(ps, 1.1, 1.1, (0, 0, 0))
    o.rebin()
    fo, _ = o.forces()
    m = o.molecules()
    expect = {1: (-24, -24, 0), 2: (24, -24, 0), 3: (-24, 24, 0), 4: (24, 24, 0)}
    for k, i in enumerate(m["ids"]):
        assert np.allclose(m["F"][k], expect[int(i)], atol=1e-8)
    assert abs(fo.upot) < 1e-8 and abs(fo.virial - 96) < 1e-8
    ps, g = golden_io.load("ref_ForceCalculationTestF0")
    o = Oracle(ps, 1.3, 1.3, (0, 0, 0))
    o.rebin()
    fo, _ = o.forces()
    assert np.abs(o.molecules()["F"]).max() < 1e-7
    assert abs(fo.upot + 4) < 1e-8 and abs(fo.virial) < 1e-6


def test_oracle_thread_count_independent():
    ps, g = golden_io.load("per_lj4000j")
    res = []
    for t in (1, 3, 8):
        o = Oracle(ps, 2.5, 2.5, (1, 1, 1), threads=t)
        o.rebin()
        fo, _ = o.forces()
        res.append((o.molecules()["F"].copy(), fo.upot))
    for F, u in res[1:]:
        assert np.array_equal(F, res[0][0])
        assert abs(u - res[0][1]) <= 1e-12 * abs(res[0][1])


@pytest.mark.parametrize("name", golden_io.names("lrc_"))
def test_oracle_longrange_homogeneous_matches_reference(name):
    """Homogeneous long-range correction (UpotCorr, VirialCorr) equal to the
    reference's own, bit for bit."""
    ps, g = golden_io.load(name)
    o = Oracle(ps, g["rc"], g["rc_lj"])
    u, w = o.longrange_homogeneous()
    assert u == float(g["upot_corr"]) and w == float(g["virial_corr"])


@pytest.mark.parametrize("name", golden_io.names("nvtt_"))
def test_oracle_velocity_scaling_thermostat_matches_reference(name):
    """NVT runs with the reference's global velocity-scaling thermostat."""
    ps, g = golden_io.load(name)
    o = Oracle(ps, g["rc"], g["rc_lj"], (1, 1, 1), threads=8)
    o.set_thermostat(float(g["target_temperature"]))
    o.rebin()
    o.forces()
    rec = o.run(float(g["dt"]), int(g["nsteps"]))
    ref = g["steps"][1:, 1:]
    for col in range(4):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-10 * scale, col
    m = o.molecules()
    a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
    for key, gk in (("r", "out_r"), ("v", "out_v"), ("q", "out_q"), ("L", "out_L")):
        assert np.abs(m[key][a] - g[gk][b]).max() < 1e-9, key
