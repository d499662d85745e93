"""Batches of independent boxes (md_batch_*) against the same boxes run one
at a time through md_ctx, and one box against the oracle.

Tolerances:
  * FP64 batch vs single-box FP64 engine: pair counts exact; Upot, virial and
    forces to 1e-10 relative (summation order differs); 40-step NVE records
    to 1e-8 relative;
  * mixed batch vs FP64 batch, after 200 FP64 steps from the generator's
    lattice sites: pair counts exact (near-cut-off pairs are re-decided in
    FP64), relative rms force error <= 1e-5 per box at rho* >= 0.3 and
    <= 1e-4 in dilute gas boxes (there the force on a molecule comes from one
    or two neighbours, often near the LJ minimum where it is the difference
    of two nearly equal terms, so FP32 coordinates weigh more), Upot to 1e-5
    relative, virial to 1e-5 of |virial| + |Upot| (the virial changes sign
    with density);
  * one box of the batch vs the oracle (the reference's algorithm): forces
    to 1e-10 relative, Upot/virial to 1e-10, pair count exact.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

RC = 2.5


@pytest.fixture(scope="module")
def mods():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine"), importlib.import_module("ls1gb300.batch")


@pytest.fixture(scope="module")
def boxes(mods):
    _, B = mods
    return B.random_boxes(6, 500, 3000, rho_range=(0.05, 0.85), seed=3)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_fp64_batch_equals_boxes_run_alone(mods, boxes):
    E, B = mods
    bt = B.Batch(boxes, RC, precision="fp64", skin=0.3)
    sums = bt.forces()
    F = bt.molecules()["F"]
    for k, bx in enumerate(boxes):
        e = E.Engine(bx.to_phasespace(rc=RC), RC, precision="fp64", skin=0.3)
        fo = e.forces()
        m = e.molecules()
        e.close()
        lo, hi = bt.box_start[k], bt.box_start[k + 1]
        assert int(sums[k, 2]) == int(fo.site_pairs[0]), k
        assert abs(sums[k, 0] - fo.upot) <= 1e-10 * abs(fo.upot), k
        assert abs(sums[k, 1] - fo.virial) <= 1e-10 * (abs(fo.virial) + abs(fo.upot)), k
        assert _rel(F[lo:hi], m["F"]) <= 1e-10, k
    bt.close()


def _evolved(B, boxes, steps=200):
    """The boxes after `steps` FP64 NVE steps: liquid- and gas-like disorder
    instead of the generator's lattice sites (where many pairs sit at the
    LJ minimum and the forces nearly cancel)."""
    bt = B.Batch(boxes, RC, precision="fp64", skin=0.3)
    bt.forces()
    bt.run(0.002, steps, record=False)
    m = bt.molecules()
    bt.close()
    out = []
    for k, b in enumerate(boxes):
        lo, hi = bt.box_start[k], bt.box_start[k + 1]
        out.append(B.Box(L=b.L, r=np.ascontiguousarray(m["r"][lo:hi]), v=np.ascontiguousarray(m["v"][lo:hi]),
                         rho=b.rho, T=b.T))
    return out


def test_mixed_batch_against_fp64_batch(mods, boxes):
    _, B = mods
    boxes = _evolved(B, boxes)
    ref = B.Batch(boxes, RC, precision="fp64", skin=0.3)
    s64 = ref.forces()
    F64 = ref.molecules()["F"]
    ref.close()
    for tpm in (1, 2, 4):
        bt = B.Batch(boxes, RC, precision="mixed", skin=0.3, threads_per_molecule=tpm)
        s32 = bt.forces()
        F32 = bt.molecules()["F"]
        bt.close()
        assert np.array_equal(s32[:, 2], s64[:, 2]), tpm
        assert np.all(np.abs(s32[:, 0] - s64[:, 0]) <= 1e-5 * np.abs(s64[:, 0])), tpm
        # the virial changes sign with density: its scale is |virial| + |Upot|
        assert np.all(np.abs(s32[:, 1] - s64[:, 1]) <= 1e-5 * (np.abs(s64[:, 1]) + np.abs(s64[:, 0]))), tpm
        for k in range(len(boxes)):
            lo, hi = bt.box_start[k], bt.box_start[k + 1]
            d = F32[lo:hi] - F64[lo:hi]
            rms = np.sqrt((d ** 2).sum(1).mean() / (F64[lo:hi] ** 2).sum(1).mean())
            assert rms <= (1e-5 if boxes[k].rho >= 0.3 else 1e-4), (tpm, k, boxes[k].rho, rms)


def test_fp64_batch_run_equals_boxes_run_alone(mods, boxes):
    """40 steps in graphs of 16 (two graph launches and a 8-step remainder)."""
    E, B = mods
    bt = B.Batch(boxes, RC, precision="fp64", skin=0.3)
    bt.forces()
    rec = bt.run(0.002, 40, graph_steps=16)
    bt.close()
    for k, bx in enumerate(boxes):
        e = E.Engine(bx.to_phasespace(rc=RC), RC, precision="fp64", skin=0.3)
        e.forces()
        r1 = e.run(0.002, 40)
        e.close()
        for col in range(3):
            assert _rel(rec[:, k, col], r1[:, col]) <= 1e-8, (k, col)


def test_batch_box_against_oracle(mods, boxes):
    _, B = mods
    bt = B.Batch(boxes, RC, precision="fp64", skin=0.0)
    sums = bt.forces()
    F = bt.molecules()["F"]
    bt.close()
    k = 2
    ps = boxes[k].to_phasespace(rc=RC)
    o = Oracle(ps, RC, threads=4)
    o.rebin()
    fo, _ = o.forces()
    om = o.molecules()
    order = np.argsort(om["ids"])
    lo, hi = bt.box_start[k], bt.box_start[k + 1]
    assert _rel(F[lo:hi], om["F"][order]) <= 1e-10
    assert abs(sums[k, 0] - fo.upot) <= 1e-10 * abs(fo.upot)
    assert abs(sums[k, 1] - fo.virial) <= 1e-10 * (abs(fo.virial) + abs(fo.upot))
    assert int(sums[k, 2]) == int(fo.site_pairs[0])


def test_autotune_picks_a_measured_configuration(mods, boxes):
    _, B = mods
    bt = B.Batch(boxes, RC, precision="mixed")
    s0 = bt.forces()
    before = bt.molecules()
    t = bt.autotune(0.002, trial_steps=8)
    after = bt.molecules()
    # the tuned configuration evaluates the same state to the same sums
    s1 = bt.forces()
    assert np.array_equal(s0[:, 2], s1[:, 2])
    assert np.allclose(s1[:, 0], s0[:, 0], rtol=1e-6, atol=0)
    assert t["trials"], t
    assert min(ms for _, _, _, ms in t["trials"]) == pytest.approx(t["ms_per_step"])
    assert (t["skin"], t["threads_per_molecule"], t["cell_occupancy"]) in [(s, p, o) for s, p, o, _ in t["trials"]]
    # the state is restored after the trials
    assert np.array_equal(before["r"], after["r"]) and np.array_equal(before["v"], after["v"])
    rec = bt.run(0.002, 20, graph_steps=10)
    assert np.all(np.isfinite(rec))
    assert np.all(rec[:, :, 2] > 0)  # every box's sum m v^2 is recorded every step
    bt.close()
