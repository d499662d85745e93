"""The reference's own mixed precision (its SPDP build: float pair
arithmetic, double accumulation) as the yardstick of the engine's mixed
precision.  Fixtures: tests/golden/spdp_*.npz (tests/golden/make_spdp.py),
one force evaluation of the reference's SPDP build on the inputs of the
periodic DPDP fixtures per_*.npz.

CPU: the reference's SPDP pair counts equal its DPDP ones, and its errors
against DPDP are those of FP32 pair arithmetic (force rms below 1e-5).
GPU: on the same inputs the engine's mixed precision -- with the rows and
with the Newton-3 forms -- is at least as close to the reference's DPDP
forces and torques as the reference's own SPDP build (within a factor 1.5,
plus a floor at FP64 rounding level; measured 1.4-4x closer with the
rows), and its Upot and virial within 5e-6 relative.  The engine's
Upot and virial totals are the less accurate ones (measured 3e-9 to 2e-6
against the SPDP build's 3e-9 to 3e-6, up to 20x apart on the 4,000-molecule
box); compensated per-molecule energy and virial sums, a Newton step on the
hardware reciprocal and exact (two-term) cell offsets were each measured and
changed none of it, so the difference lies elsewhere in the FP32 pair
arithmetic (not isolated); the forces, which carry the dynamics, are the
more accurate ones."""
import numpy as np
import pytest

import golden_io as G

CASES = ["lj500", "lj4000j", "lj864_rclj", "mix500", "slab"]


def _rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum(1).mean() / (b ** 2).sum(1).mean()))


def _spdp(case):
    z = np.load(f"{G.GOLDEN}/spdp_{case}.npz")
    ps, g = G.load(str(z["input"]))
    np.testing.assert_array_equal(z["out_ids"], g["out_ids"])
    return ps, g, z


def _errors(F, M, upot, virial, g):
    e = {"F": _rms(F, g["F"]), "upot": abs(upot - float(g["upot"])) / abs(float(g["upot"])),
         "virial": abs(virial - float(g["virial"])) / abs(float(g["virial"]))}
    if np.abs(g["M"]).max() > 0:
        e["M"] = _rms(M, g["M"])
    return e


@pytest.mark.parametrize("case", CASES)
def test_reference_spdp_error_against_its_dpdp(case):
    ps, g, z = _spdp(case)
    np.testing.assert_array_equal(z["counts"], g["counts"])
    e = _errors(z["F"], z["M"], float(z["upot"]), float(z["virial"]), g)
    assert 0 < e["F"] < 1e-5, e
    assert e["upot"] < 1e-5 and e["virial"] < 1e-5, e


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["rows", "newton3"])
@pytest.mark.parametrize("case", CASES)
def test_engine_mixed_at_least_as_close_as_the_reference_spdp(case, scheme):
    """Both pair schemes: the rows, and the Newton-3 forms (cluster pairs for
    single-centre LJ with rc_lj = rc, half rows with atomics for the
    mixture; every one of these boxes has three list cells per axis at skin
    0, and the case with rc_lj < rc runs on the rows)."""
    import build as eb
    eb.build()
    from ls1gb300 import engine as E
    ps, g, z = _spdp(case)
    ref = _errors(z["F"], z["M"], float(z["upot"]), float(z["virial"]), g)
    e = E.Engine(ps, g["rc"], g["rc_lj"], precision="mixed", pair_scheme=scheme)
    fo = e.forces()
    m = e.molecules()
    n3 = scheme == "newton3" and (case == "mix500" or float(g["rc_lj"]) == float(g["rc"]))
    assert e.time_kernels(1).pair_scheme == (1 if n3 else 0)
    e.close()
    o = np.argsort(m["ids"])
    got = _errors(m["F"][o], m["M"][o], fo.upot, fo.virial, g)
    table = {k: (got[k], ref[k]) for k in ref}
    for k in ("F", "M"):
        if k in ref:
            assert got[k] <= 1.5 * ref[k] + 1e-7, (k, table)
    for k in ("upot", "virial"):
        assert got[k] <= 5e-6, (k, table)
