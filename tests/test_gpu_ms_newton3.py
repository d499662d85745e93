"""The multi-site kernels' Newton-3 form (md_config.pair_scheme =
MD_PAIRS_NEWTON3, mixed precision): every molecule pair is evaluated once,
from the higher-slot part of the lower slot's candidate row, and the
neighbour's force, torque and virial are added to FP32 accumulators by
vector atomics (Newton's third law as the reference's processCellPair
applies it, VectorizedCellProcessor.cpp:2744-2819).

Bars:
  * against the reference's golden outputs of every multi-site case (the
    ten Vectorization inputs, nine of them multi-site, and the periodic
    mixture): the mixed tolerances of the row kernels (relative rms force
    error <= 1e-5, torques and virials <= 1e-4, Upot/virial 1e-5), site pair
    counts exact;
  * against the rows (every pair from both sides) on the same state:
    molecule and site pair counts equal, F, M, Vi to 1e-5 relative rms (two
    FP32 summation orders), Upot and virial to 1e-6 relative;
  * the reference's NVE run of the rotating mixture (nve_mix500, 20 steps):
    per-step Upot, virial, sum m v^2, sum I w^2 to 1e-4 relative, the mixed
    NVE tolerance;
  * md_adjoint on a Newton-3 context (its own Newton-3 kernel: each pair
    once, the neighbour's position gradient by atomics) equals the rows
    context's to 1e-5, with and without a force cotangent;
  * edge cases against the oracle (one molecule, a pair across the periodic
    boundary, a dilute gas, a dense block in a corner of a large box and in
    a closed box): pair counts exact, forces 1e-5 rms, torques 1e-4.
"""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


def _multisite(ps):
    return any(len(c.lj) != 1 or c.charges or c.dipoles or c.quadrupoles or any(x != 0 for x in c.lj[0].r)
               for c in ps.components)


MS_CASES = [n for n in golden_io.names("ref_") + golden_io.names("per_") if _multisite(golden_io.load(n)[0])]


@pytest.fixture(scope="module")
def E():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def _by_id(ids):
    return np.argsort(ids, kind="stable")


def _rel_rms(a, b):
    return np.sqrt(((a - b) ** 2).sum(axis=1).mean()) / max(np.sqrt((b ** 2).sum(axis=1).mean()), 1e-300)


def _run(E, ps, g, scheme):
    e = E.Engine(ps, g["rc"], g["rc_lj"], (1, 1, 1) if g["periodic"] else (0, 0, 0), precision="mixed", skin=0.0,
                 pair_scheme=scheme)
    fo = e.forces()
    m = e.molecules()
    used = e.time_kernels(1).pair_scheme
    return e, fo, m, used


def test_the_multisite_cases_are_there():
    assert len(MS_CASES) == 10 and "per_mix500" in MS_CASES


@pytest.mark.parametrize("name", MS_CASES)
def test_newton3_forces_match_reference_and_rows(E, name):
    ps, g = golden_io.load(name)
    e, fo, m, used = _run(E, ps, g, "newton3")
    e.close()
    assert used == 1
    a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
    assert _rel_rms(m["F"][a], g["F"][b]) <= 1e-5
    for key in ("M", "Vi"):
        if np.abs(g[key]).max() > 1e-6:
            assert _rel_rms(m[key][a], g[key][b]) <= 1e-4, key
        else:
            assert np.abs(m[key][a] - g[key][b]).max() < 1e-4, key
    for mine, ref in ((fo.upot, float(g["upot"])), (fo.virial, float(g["virial"]))):
        assert abs(mine - ref) <= 1e-5 * max(1.0, abs(ref))
    assert list(fo.site_pairs) == list(g["counts"][2::2].astype(np.int64))
    # the rows on the same state
    er, fr, mr, used_r = _run(E, ps, g, "rows")
    er.close()
    assert used_r == 0
    assert fo.mol_pairs == fr.mol_pairs and list(fo.site_pairs) == list(fr.site_pairs)
    ia, ir = _by_id(m["ids"]), _by_id(mr["ids"])
    for key in ("F", "M", "Vi"):
        if np.abs(mr[key]).max() > 1e-6:
            assert _rel_rms(m[key][ia], mr[key][ir]) <= 1e-5, key
        else:
            assert np.abs(m[key][ia] - mr[key][ir]).max() < 1e-6, key
    assert abs(fo.upot - fr.upot) <= 1e-6 * abs(fr.upot)
    assert abs(fo.virial - fr.virial) <= 1e-6 * max(abs(fr.virial), 1e-300)


def test_newton3_nve_of_the_rotating_mixture(E):
    ps, g = golden_io.load("nve_mix500")
    e = E.Engine(ps, g["rc"], g["rc_lj"], (1, 1, 1), precision="mixed", skin=0.0, pair_scheme="newton3")
    e.forces()
    rec = e.run(float(g["dt"]), int(g["nsteps"]))
    assert e.time_kernels(1).pair_scheme == 1
    e.close()
    ref = g["steps"][1:, 1:]
    for col in range(4):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-4 * scale, col


@pytest.mark.parametrize("with_gF", [False, True])
@pytest.mark.parametrize("name", ["per_mix500", "ref_VectorizationDipoleQuadrupole",
                                  "ref_VectorizationMultiComponentMultiPotentials"])
def test_adjoint_on_a_newton3_context_equals_the_rows(E, name, with_gF):
    """md_adjoint on a Newton-3 context runs its Newton-3 kernel (each pair
    once, the neighbour's share by atomics): the same position and
    parameter gradients as the rows context's adjoint (every pair from both
    sides) to 1e-5 -- with and without a force cotangent gF (the dual-number
    and the homogeneity instances), for the two-component kernel and the
    general one."""
    ps, g = golden_io.load(name)
    gF = np.random.default_rng(3).normal(size=(ps.n, 3)) if with_gF else None
    out = {}
    for scheme in ("newton3", "rows"):
        e, fo, m, used = _run(E, ps, g, scheme)
        gr, gp = e.adjoint(1.0, 0.5, gF)
        e.close()
        out[scheme] = (gr, gp, used)
    assert out["newton3"][2] == 1 and out["rows"][2] == 0
    gr3, gp3, _ = out["newton3"]
    grr, gpr, _ = out["rows"]
    # grad_r is in upload order in both contexts
    assert _rel_rms(gr3, grr) <= 1e-5
    assert np.abs(gp3 - gpr).max() <= 1e-5 * np.abs(gpr).max()


def _subset(ps0, idx, box, r):
    """Molecules idx of ps0 at positions r in a box of edge box."""
    q = ps0.copy()
    idx = np.asarray(idx)
    q.box = np.array([box, box, box], float)
    q.ids, q.comp = ps0.ids[idx].copy(), ps0.comp[idx].copy()
    q.r = np.asarray(r, float).reshape(len(idx), 3)
    q.v, q.q, q.L = ps0.v[idx].copy(), ps0.q[idx].copy(), ps0.L[idx].copy()
    return q


def _edge_cases():
    from ls1gb300 import phasespace as psm
    ps0 = psm.mixture(500, 18.0, 300.0, seed=9)
    a0, b0 = int(np.flatnonzero(ps0.comp == 0)[0]), int(np.flatnonzero(ps0.comp == 1)[0])
    rng = np.random.default_rng(17)
    pts = []
    while len(pts) < 40:
        p = rng.uniform(0, 10.0, 3)
        if all(np.linalg.norm(((p - q) + 5.0) % 10.0 - 5.0) > 0.6 for q in pts):
            pts.append(p)
    return {
        "single": (_subset(ps0, [a0], 4.0, [[2.0, 2.0, 2.0]]), (1, 1, 1)),
        # an A and a B molecule 0.55 nm apart across the periodic boundary
        "pair_across_boundary": (_subset(ps0, [a0, b0], 4.0, [[0.2, 2.0, 2.0], [3.65, 2.05, 1.95]]), (1, 1, 1)),
        # 40 molecules in a 10 nm box: mostly empty cells, most half rows empty
        "dilute": (_subset(ps0, np.arange(40), 10.0, pts), (1, 1, 1)),
        # the 500-molecule block in a corner of a 9 nm box, wrapped across the boundary: long rows
        "corner_cluster": (_subset(ps0, np.arange(ps0.n), 9.0, np.mod(ps0.r - 1.0, 9.0)), (1, 1, 1)),
        # the same block in a closed (non-periodic) box
        "closed_box": (_subset(ps0, np.arange(ps0.n), 6.5, ps0.r + 1.5), (0, 0, 0)),
    }


EDGE = sorted(_edge_cases())


@pytest.mark.parametrize("name", EDGE)
def test_newton3_edge_cases_against_the_oracle(E, name):
    """Edge cases of the half rows and the cross-molecule ring against the
    oracle (FP64, the reference's algorithm): one molecule, a pair across
    the periodic boundary, a dilute gas (most half rows empty, warps with
    few in-cut-off pairs), a dense block in one corner of a large box (long
    rows) and in a closed box.  Pair counts exact, relative rms force error
    <= 1e-5, torques <= 1e-4, Upot and virial <= 1e-5 relative."""
    from oracle.oracle import Oracle
    ps, per = _edge_cases()[name]
    e = E.Engine(ps, 1.0, 1.0, per, precision="mixed", skin=0.3, pair_scheme="newton3")
    fo = e.forces()
    m = e.molecules()
    assert e.time_kernels(1).pair_scheme == 1
    e.close()
    o = Oracle(ps, 1.0, 1.0, per)
    o.rebin()
    foo, _ = o.forces()
    mo = o.molecules()
    assert fo.mol_pairs == foo.mol_pairs and list(fo.site_pairs) == list(foo.site_pairs)
    a, b = _by_id(m["ids"]), _by_id(mo["ids"])
    for key, tol in (("F", 1e-5), ("M", 1e-4)):
        if np.abs(mo[key]).max() > 0:
            assert _rel_rms(m[key][a], mo[key][b]) <= tol, key
        else:
            assert np.abs(m[key]).max() == 0.0, key
    for mine, ref in ((fo.upot, foo.upot), (fo.virial, foo.virial)):
        assert abs(mine - ref) <= 1e-5 * max(abs(ref), 1e-300) or (ref == 0.0 and mine == 0.0)
