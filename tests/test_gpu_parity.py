"""Parity of the CUDA engine (through the C ABI) with the reference's golden
outputs and with the pinned C oracle.

Tolerances:
  * cell assignment, halo copy count, largest cell occupancy and the
    interacting molecule / site pair counts: exact, in both precisions (the
    mixed kernel re-decides pairs within 4e-6 relative of the cut-off in FP64);
  * FP64 kernel: F, M, Vi and Upot/virial to 1e-10 relative to the largest
    magnitude of the case (FMA contraction and summation order differ);
  * mixed kernel: relative rms force error <= 1e-5 (the precision target
    stated for this path), torques and virials <= 1e-4, Upot/virial 1e-5;
  * NVE runs (md_run, CUDA graph): per-step Upot, virial, sum m v^2 and
    sum I w^2 to 1e-8 relative (FP64), 1e-4 (mixed, 10-20 steps).
"""
import numpy as np
import pytest

import golden_io
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

FORCE_CASES = golden_io.names("ref_") + golden_io.names("per_")
NVE_CASES = golden_io.names("nve_")


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import sys
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "ls1-mardyn_gb300"))
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def _by_id(ids):
    return np.argsort(ids, kind="stable")


def _rel_max(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _rel_rms(a, b):
    return np.sqrt(((a - b) ** 2).sum(axis=1).mean()) / max(np.sqrt((b ** 2).sum(axis=1).mean()), 1e-300)


def _engine(E, name, precision, skin=0.0):
    ps, g = golden_io.load(name)
    e = E.Engine(ps, g["rc"], g["rc_lj"], (1, 1, 1) if g["periodic"] else (0, 0, 0), precision=precision, skin=skin)
    return ps, g, e


@pytest.mark.parametrize("name", FORCE_CASES)
def test_fp64_forces_match_reference(engine_mod, name):
    ps, g, e = _engine(engine_mod, name, "fp64")
    st = e.rebin()
    assert list(st.cells) == list(g["grid"])
    o = Oracle(ps, g["rc"], g["rc_lj"], (1, 1, 1) if g["periodic"] else (0, 0, 0))
    ost = o.rebin()
    assert st.n_halo == ost.n_halo
    assert st.max_occupancy == ost.max_occupancy
    fo = e.forces()
    m = e.molecules()
    a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
    assert np.array_equal(m["ids"][a], g["out_ids"][b])
    assert np.array_equal(e.cells()[a], g["out_cell"][b])
    for key in ("F", "M", "Vi"):
        # forces that cancel to rounding level (ForceCalculationTestF0) are
        # compared in absolute terms, as the reference's own test does
        scale = max(np.abs(g[key]).max(), 1.0)
        assert np.abs(m[key][a] - g[key][b]).max() <= 1e-10 * scale, key
    for mine, ref in ((fo.upot, float(g["upot"])), (fo.virial, float(g["virial"]))):
        assert abs(mine - ref) <= 1e-10 * max(1.0, abs(ref))
    assert list(fo.site_pairs) == list(g["counts"][2::2].astype(np.int64))
    ofo, _ = o.forces()
    assert fo.mol_pairs == ofo.mol_pairs


@pytest.mark.parametrize("name", FORCE_CASES)
def test_mixed_forces_match_reference(engine_mod, name):
    ps, g, e = _engine(engine_mod, name, "mixed")
    e.rebin()
    fo = e.forces()
    m = e.molecules()
    a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
    if np.abs(g["F"]).max() > 1e-6:
        assert _rel_rms(m["F"][a], g["F"][b]) <= 1e-5
    else:
        assert np.abs(m["F"] - g["F"]).max() < 1e-4
    for key in ("M", "Vi"):
        if np.abs(g[key]).max() > 1e-6:
            assert _rel_rms(m[key][a], g[key][b]) <= 1e-4, key
        else:
            assert np.abs(m[key][a] - g[key][b]).max() < 1e-4, key
    for mine, ref in ((fo.upot, float(g["upot"])), (fo.virial, float(g["virial"]))):
        assert abs(mine - ref) <= 1e-5 * max(1.0, abs(ref))
    assert list(fo.site_pairs) == list(g["counts"][2::2].astype(np.int64))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", NVE_CASES)
def test_nve_matches_reference(engine_mod, name, precision):
    ps, g = golden_io.load(name)
    skin = 0.3 * g["rc"] if precision == "mixed" else 0.0
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], (1, 1, 1), precision=precision, skin=skin)
    e.forces()
    rec = e.run(float(g["dt"]), int(g["nsteps"]))
    ref = g["steps"][1:, 1:]
    tol = 1e-8 if precision == "fp64" else 1e-4
    for col in range(4):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= tol * scale, col
    if precision == "fp64" and "out_r" in g:
        m = e.molecules()
        a, b = _by_id(m["ids"]), _by_id(g["out_ids"])
        for key, gk in (("r", "out_r"), ("v", "out_v"), ("q", "out_q"), ("L", "out_L")):
            assert np.abs(m[key][a] - g[gk][b]).max() < 1e-7, key


@pytest.mark.parametrize("name", NVE_CASES)
def test_newton3_nve_matches_reference(engine_mod, name):
    """The Newton-3 cluster-pair path (mixed precision, every pair once) over
    the reference's NVE runs, to the mixed tolerance (1e-4 on the per-step
    sums), where the box allows it (one component of single-centre LJ
    molecules, three list cells per axis); other cases use the rows."""
    ps, g = golden_io.load(name)
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], (1, 1, 1), precision="mixed", skin=0.3 * g["rc"],
                          pair_scheme="newton3")
    e.forces()
    rec = e.run(float(g["dt"]), int(g["nsteps"]))
    ref = g["steps"][1:, 1:]
    for col in range(4):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-4 * scale, col


def test_skin_does_not_change_the_trajectory(engine_mod):
    """The pair-candidate list with a skin finds exactly the pairs of the
    rebuild-every-step schedule: FP64 runs with skin 0 and skin 0.4 agree."""
    ps, g = golden_io.load("per_lj4000j")
    runs = []
    for skin in (0.0, 0.4):
        e = engine_mod.Engine(ps, 2.5, 2.5, precision="fp64", skin=skin)
        e.forces()
        runs.append(e.run(0.002, 60))
    assert np.abs(runs[0] - runs[1]).max() <= 1e-9 * np.abs(runs[0]).max()


def test_step_by_step_equals_md_run(engine_mod):
    """md_integrate_pre / md_compute_forces / md_integrate_post (the
    Leapfrog/ParticleContainer mirror) equal the graph-captured md_run."""
    ps, g = golden_io.load("per_lj500")
    cells = engine_mod.GpuLinkedCells(ps, 2.5, precision="fp64", skin=0.3)
    lf = engine_mod.GpuLeapfrog(0.002)
    cells.traverseCells()
    manual = []
    for _ in range(12):
        lf.eventNewTimestep(cells)
        fo = cells.traverseCells()
        ko = lf.eventForcesCalculated(cells)
        manual.append([fo.upot, fo.virial, ko.summv2])
    e = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.3)
    e.forces()
    rec = e.run(0.002, 12)
    assert np.allclose(np.array(manual), rec[:, :3], rtol=1e-12, atol=0)


@pytest.mark.parametrize("scheme", ["rows", "newton3"])
def test_fused_leapfrog_steps_equal_step_by_step(engine_mod, scheme):
    """Mixed precision, one component of single-centre LJ molecules: md_run
    runs Leapfrog's post-force half step of each step and the pre-force half
    step of the next with the pair evaluation -- in the row kernel's epilogue
    (two position buffers) with per-molecule rows, in k_n3_lf after the
    Newton-3 pair kernel with cluster pairs.  60 steps (two graph-captured
    chunks and an eager remainder, several list rebuilds) against
    md_integrate_pre / md_compute_forces / md_integrate_post.  Rows: the same
    FP64 operations, so positions, velocities, Upot and virial agree bit for
    bit, the kinetic sums (FP32 products in the fused kernel) to 1e-6.
    Cluster pairs: the force accumulators take their atomic additions in an
    arbitrary order, so both runs agree to FP32 rounding carried over 60
    steps: Upot, virial and kinetic sums to 1e-5, positions to 1e-5."""
    ps, g = golden_io.load("per_lj500")
    rng = np.random.default_rng(5)
    ps.v = ps.v * 1.5 + rng.normal(0.0, 0.2, ps.v.shape)
    cells = engine_mod.GpuLinkedCells(ps, 2.5, precision="mixed", skin=0.2, pair_scheme=scheme)
    lf = engine_mod.GpuLeapfrog(0.004)
    cells.traverseCells()
    manual = []
    for _ in range(60):
        lf.eventNewTimestep(cells)
        fo = cells.traverseCells()
        ko = lf.eventForcesCalculated(cells)
        manual.append([fo.upot, fo.virial, ko.summv2])
    manual = np.array(manual)
    e = engine_mod.Engine(ps, 2.5, precision="mixed", skin=0.2, pair_scheme=scheme)
    e.forces()
    rec = e.run(0.004, 60)
    a, b = cells.molecules(), e.molecules()
    assert e.rebuilds() >= 3
    assert e.time_kernels(1).pair_scheme == (1 if scheme == "newton3" else 0)
    e.close()
    if scheme == "rows":
        np.testing.assert_array_equal(rec[:, :2], manual[:, :2])
        assert np.abs(rec[:, 2] - manual[:, 2]).max() <= 1e-6 * np.abs(manual[:, 2]).max()
        for k in ("ids", "r", "v", "F"):
            np.testing.assert_array_equal(a[k], b[k])
        return
    for col in range(3):
        assert np.abs(rec[:, col] - manual[:, col]).max() <= 1e-5 * np.abs(manual[:, col]).max(), col
    ia, ib = _by_id(a["ids"]), _by_id(b["ids"])
    assert np.abs(a["r"][ia] - b["r"][ib]).max() <= 1e-5


@pytest.mark.parametrize("name", ["per_lj4000j", "nve_lj32000", "per_lj500"])
def test_cluster_pairs_match_candidate_rows(engine_mod, name):
    """Mixed precision: the Newton-3 cluster-pair path (every pair once) and
    the per-molecule candidate rows (every pair from both sides) on the same
    state: interacting pair counts equal, forces and per-molecule virials to
    1e-6 relative rms, Upot and virial to 1e-6 relative; and boxes with fewer
    than three list cells along a periodic axis fall back to the rows."""
    ps, g = golden_io.load(name)
    rng = np.random.default_rng(11)
    ps.r = ps.r + rng.uniform(-0.05, 0.05, ps.r.shape)
    out = {}
    for scheme in ("newton3", "rows"):
        e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="mixed", skin=0.25, pair_scheme=scheme)
        fo = e.forces()
        m = e.molecules()
        out[scheme] = (fo, m, e.time_kernels(1).pair_scheme)
        e.close()
    assert out["newton3"][2] == 1 and out["rows"][2] == 0
    fa, ma, _ = out["newton3"]
    fr, mr, _ = out["rows"]
    assert fa.mol_pairs == fr.mol_pairs and list(fa.site_pairs) == list(fr.site_pairs)
    ia, ir = _by_id(ma["ids"]), _by_id(mr["ids"])
    assert _rel_rms(ma["F"][ia], mr["F"][ir]) <= 1e-6
    assert _rel_rms(ma["Vi"][ia], mr["Vi"][ir]) <= 1e-6
    assert np.all(ma["M"] == 0.0)
    assert abs(fa.upot - fr.upot) <= 1e-6 * abs(fr.upot)
    assert abs(fa.virial - fr.virial) <= 1e-6 * abs(fr.virial)
    # a box of 2 x 2 x 2 list cells: rows
    small = psm_small()
    e = engine_mod.Engine(small, 2.5, precision="mixed", skin=0.25, pair_scheme="newton3")
    e.forces()
    assert e.time_kernels(1).pair_scheme == 0
    e.close()


def psm_small():
    from ls1gb300 import phasespace as psm
    return psm.lj_fcc(4, 0.8, 1.0, seed=3)   # L = 6.84: two list cells of edge >= 2.75 per axis


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reupload_with_set_forces_continues_the_run(engine_mod, precision):
    """A caller that downloads, edits nothing and re-uploads the molecules
    between the force evaluation and the next pre-force half step (ls1's
    host mirror after a plugin iterated it) hands the forces back with
    md_set_forces; the step that follows equals the one without the round
    trip (FP64: bit for bit)."""
    ps, g = golden_io.load("per_mix500")
    a = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision=precision)
    b = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision=precision)
    dt = 5e-5
    for e in (a, b):
        e.forces()
        e.pre(dt)
        e.forces()
        e.post(dt)
    m = b.molecules()
    q = ps.copy()
    o = _by_id(m["ids"])
    q.r, q.v, q.q, q.L, q.ids, q.comp = m["r"][o], m["v"][o], m["q"][o], m["L"][o], m["ids"][o], m["comp"][o]
    b.upload(q)
    b.set_forces(m["F"][o], m["M"][o], m["Vi"][o])
    for e in (a, b):
        e.pre(dt)
        e.forces()
        e.post(dt)
    ma, mb = a.molecules(), b.molecules()
    a.close()
    b.close()
    ia, ib = _by_id(ma["ids"]), _by_id(mb["ids"])
    for k in ("r", "v", "q", "L", "F"):
        if precision == "fp64":
            np.testing.assert_array_equal(ma[k][ia], mb[k][ib], k)
        else:
            assert np.abs(ma[k][ia] - mb[k][ib]).max() <= 1e-6 * max(np.abs(ma[k]).max(), 1e-300), k


def test_mixed_matches_fp64_at_scale(engine_mod):
    """1CLJ N=32000 (the reference's small benchmark case): mixed-precision
    forces within 1e-5 relative rms of the FP64 kernel, Upot within 1e-6."""
    ps, g = golden_io.load("nve_lj32000")
    rng = np.random.default_rng(3)
    ps.r = ps.r + rng.uniform(-0.1, 0.1, ps.r.shape)
    out = {}
    for prec in ("fp64", "mixed"):
        e = engine_mod.Engine(ps, 2.5, precision=prec, skin=0.3)
        fo = e.forces()
        out[prec] = (e.molecules()["F"], fo)
    assert _rel_rms(out["mixed"][0], out["fp64"][0]) <= 1e-5
    assert abs(out["mixed"][1].upot - out["fp64"][1].upot) <= 1e-6 * abs(out["fp64"][1].upot)
    assert out["mixed"][1].site_pairs[0] == out["fp64"][1].site_pairs[0]
