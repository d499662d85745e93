"""Edge cases of the binning, the candidate list and the pair kernels,
engine against the oracle (the reference's algorithm) on the same inputs:
one molecule, an isolated pair across the periodic boundary, a dilute gas
with mostly empty cells, a dense cluster in one corner of a large box (long
candidate rows: the list capacity has to grow), closed (non-periodic)
boundaries, and a run through all of them.

Tolerances: FP64 forces, Upot and virial to 1e-10 relative (the engine sums
in another order); pair counts exact; mixed precision: relative rms force
error 1e-5 and exact pair counts.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def _ps(box, r, v=None, seed=0):
    from ls1gb300 import phasespace as psm
    n = len(r)
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3)) if v is None else np.asarray(v, float)
    q = np.zeros((n, 4))
    q[:, 0] = 1.0
    return psm.PhaseSpace(np.asarray(box, float), [psm.one_center_lj()], [], 1.0e10,
                          np.arange(1, n + 1, dtype=np.uint64), np.zeros(n, np.int32), np.asarray(r, float), v, q,
                          np.zeros((n, 3)), 1.0)


def _cases():
    rng = np.random.default_rng(42)
    out = {"single": (_ps([9.0, 9.0, 9.0], [[4.5, 4.5, 4.5]]), 2.5, (1, 1, 1)),
           # r = 0.96 (repulsive): away from the LJ minimum at 1.12, where the force of one isolated pair is the
           # difference of two nearly equal terms and its FP32 relative error is not a measure of the kernel
           "pair_across_boundary": (_ps([10.0, 10.0, 10.0], [[0.3, 5.0, 5.0], [9.35, 5.1, 4.9]]), 2.5, (1, 1, 1))}
    # dilute gas: 60 molecules in a box of 40^3 (mostly empty cells), no overlaps below 1.0
    pts = []
    while len(pts) < 60:
        p = rng.uniform(0, 40, 3)
        if all(np.linalg.norm(((p - q) + 20) % 40 - 20) > 1.0 for q in pts):
            pts.append(p)
    out["dilute"] = (_ps([40.0, 40.0, 40.0], pts, seed=1), 2.5, (1, 1, 1))
    # dense cluster: an fcc block of 864 molecules at rho* = 0.9 in one corner of a 30^3 box
    from ls1gb300 import phasespace as psm
    a = (4 / 0.9) ** (1 / 3)
    blk = psm.fcc_positions((6, 6, 6), a) + rng.uniform(-0.05, 0.05, (864, 3))
    out["corner_cluster"] = (_ps([30.0, 30.0, 30.0], np.mod(blk - 1.0, 30.0), seed=2), 2.5, (1, 1, 1))
    # closed boundaries: the same block in the middle of a box without periodic images
    out["closed_box"] = (_ps([20.0, 20.0, 20.0], blk + 5.0, seed=3), 2.5, (0, 0, 0))
    out["slab_periodic_xy"] = (_ps([11.0, 11.0, 30.0], np.mod(blk, [11.0, 11.0, 30.0]) + [0, 0, 8.0], seed=4), 2.5,
                               (1, 1, 0))
    return out


CASES = _cases()


def _oracle(ps, rc, per):
    o = Oracle(ps, rc, rc, per, threads=4)
    o.rebin()
    fo, _ = o.forces()
    m = o.molecules()
    order = np.argsort(m["ids"])
    return fo, m["F"][order]


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_forces_match_oracle(engine_mod, name):
    ps, rc, per = CASES[name]
    fo_ref, F_ref = _oracle(ps, rc, per)
    for skin in (0.0, 0.4):
        e = engine_mod.Engine(ps, rc, precision="fp64", periodic=per, skin=skin)
        fo = e.forces()
        m = e.molecules()
        e.close()
        order = np.argsort(m["ids"])
        scale = max(np.abs(F_ref).max(), 1e-300)
        assert np.abs(m["F"][order] - F_ref).max() <= 1e-10 * scale, skin
        assert abs(fo.upot - fo_ref.upot) <= 1e-10 * max(abs(fo_ref.upot), 1e-300), skin
        assert abs(fo.virial - fo_ref.virial) <= 1e-10 * max(abs(fo_ref.virial), 1e-300), skin
        assert int(fo.site_pairs[0]) == int(fo_ref.site_pairs[0]), skin
        assert int(fo.mol_pairs) == int(fo_ref.mol_pairs), skin


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_forces_match_oracle(engine_mod, name):
    ps, rc, per = CASES[name]
    fo_ref, F_ref = _oracle(ps, rc, per)
    e = engine_mod.Engine(ps, rc, precision="mixed", periodic=per, skin=0.3)
    fo = e.forces()
    m = e.molecules()
    e.close()
    assert int(fo.site_pairs[0]) == int(fo_ref.site_pairs[0])
    F = m["F"][np.argsort(m["ids"])]
    if np.abs(F_ref).max() == 0.0:
        assert np.all(F == 0.0)
    else:
        rms = np.sqrt(((F - F_ref) ** 2).sum(1).mean() / (F_ref ** 2).sum(1).mean())
        assert rms <= 1e-5
    assert abs(fo.upot - fo_ref.upot) <= 1e-5 * max(abs(fo_ref.upot), 1e-300)


@pytest.mark.parametrize("name", sorted(CASES))
def test_runs_match_oracle(engine_mod, name):
    """20 NVE steps (FP64, list skin 0.4) against the oracle's run."""
    ps, rc, per = CASES[name]
    o = Oracle(ps, rc, rc, per, threads=4)
    o.rebin()
    o.forces()
    ref = o.run(0.002, 20)
    e = engine_mod.Engine(ps, rc, precision="fp64", periodic=per, skin=0.4)
    e.forces()
    rec = e.run(0.002, 20)
    e.close()
    for col in range(3):
        scale = max(np.abs(ref[:, col]).max(), 1e-300)
        assert np.abs(rec[:, col] - ref[:, col]).max() <= 1e-9 * scale, col
