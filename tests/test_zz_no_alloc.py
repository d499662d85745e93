"""The allocation-free entry point md_forces_lj_noalloc, for callers that
cannot allocate device memory (graphs owned by a larger application, pooled
device memory, real-time drivers): called twice in a row through the C ABI
on device buffers the caller owns, it must reproduce the forces, Upot and
virial of the regular entry point (md_compute_forces, FP64) and of the
oracle to 1e-10 relative -- with positions outside [0, L), exactly on 0 and
L, on a non-default stream, at three cells per axis and at its molecule
limit; oversize requests are rejected before any device work.
This file is collected last on purpose."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
sys.path.insert(0, ROOT)

pytestmark = pytest.mark.gpu

MD_ERR_CAPACITY, MD_ERR_UNSUPPORTED = 3, 6


def _setup():
    import build as eb
    eb.build()
    from ls1gb300 import engine as E
    from ls1gb300 import phasespace as psm
    L = E.load_library()
    L.md_forces_lj_noalloc.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    L.md_forces_lj_noalloc.restype = C.c_int
    return E, psm, L


def _regular(E, ps, rc):
    """Forces, Upot and virial of the regular FP64 entry point on wrapped positions."""
    q = ps.copy()
    q.r = np.mod(q.r, q.box)
    q.r[q.r >= q.box] = 0.0
    e = E.Engine(q, rc, precision="fp64")
    fo = e.forces()
    F = e.molecules()["F"]
    e.close()
    return F, fo.upot, fo.virial


def _oracle(ps, rc):
    from oracle.oracle import Oracle
    q = ps.copy()
    q.r = np.mod(q.r, q.box)
    q.r[q.r >= q.box] = 0.0
    o = Oracle(q, rc, threads=os.cpu_count() or 1)
    o.rebin()
    fo, _ = o.forces()
    return o.molecules()["F"], fo.upot, fo.virial


def _noalloc_twice(L, ps, rc, F_ref, u_ref, w_ref, stream=None):
    import torch
    r = torch.tensor(ps.r, dtype=torch.float64, device="cuda")
    F = torch.empty_like(r)
    uv = torch.empty(2, dtype=torch.float64, device="cuda")
    box = (C.c_double * 3)(*ps.box)
    sp = None if stream is None else stream.cuda_stream
    for _ in range(2):
        F.fill_(float("nan"))
        uv.fill_(float("nan"))
        torch.cuda.synchronize()
        rc_ = L.md_forces_lj_noalloc(r.data_ptr(), ps.n, box, rc, 1.0, 1.0, 0.0, F.data_ptr(), uv.data_ptr(), sp)
        torch.cuda.synchronize()
        assert rc_ == 0
        Fn = F.cpu().numpy()
        assert np.abs(Fn - F_ref).max() <= 1e-10 * np.abs(F_ref).max()
        u, w = uv.cpu().numpy()
        assert abs(u - u_ref) <= 1e-10 * abs(u_ref)
        assert abs(w - w_ref) <= 1e-10 * abs(w_ref)


def test_noalloc_matches_regular_entry_point_twice():
    pytest.importorskip("torch")
    E, psm, L = _setup()
    ps = psm.lj_fcc(8, 0.8, 1.0, seed=13)
    ps.r = ps.r + np.random.default_rng(13).uniform(-0.12, 0.12, ps.r.shape)
    ps.r = np.mod(ps.r, ps.box)
    rc = 2.5
    _noalloc_twice(L, ps, rc, *_regular(E, ps, rc))


def test_noalloc_unwrapped_positions_on_a_side_stream():
    """Positions shifted by +-L (and some exactly on 0 and L) are binned and
    paired by the kernel's own periodic images; the call runs on a
    non-default stream."""
    torch = pytest.importorskip("torch")
    E, psm, L = _setup()
    ps = psm.lj_fcc(7, 0.8, 1.0, seed=21)
    rng = np.random.default_rng(21)
    ps.r = np.mod(ps.r + rng.uniform(-0.1, 0.1, ps.r.shape), ps.box)
    ps.r[np.argsort(ps.r[:, 0])[:3], 0] = 0.0            # the three nearest the lower x face onto it
    ps.r[np.argsort(-ps.r[:, 1])[:3], 1] = ps.box[1]     # the three nearest the upper y face onto it
    sel = rng.random(ps.r.shape) < 0.3
    ps.r = ps.r + np.where(sel, rng.choice([-1.0, 1.0], ps.r.shape), 0.0) * ps.box
    rc = 2.5
    ref = _regular(E, ps, rc)
    s = torch.cuda.Stream()
    _noalloc_twice(L, ps, rc, *ref, stream=s)


def test_noalloc_three_cells_per_axis_against_the_oracle():
    pytest.importorskip("torch")
    E, psm, L = _setup()
    ps = psm.lj_fcc(5, 0.8, 1.0, seed=5)   # L = 8.55: three cells of edge >= 2.5 per axis
    ps.r = np.mod(ps.r + np.random.default_rng(5).uniform(-0.15, 0.15, ps.r.shape), ps.box)
    rc = 2.5
    assert int(ps.box[0] / rc) == 3
    _noalloc_twice(L, ps, rc, *_oracle(ps, rc))


def test_noalloc_at_its_molecule_limit_against_the_oracle():
    pytest.importorskip("torch")
    E, psm, L = _setup()
    ps = psm.lj_fcc(32, 0.8, 1.0, seed=32)  # 131,072 molecules = MD_NOALLOC_MAX_N
    assert ps.n == 131072
    ps.r = np.mod(ps.r + np.random.default_rng(32).uniform(-0.1, 0.1, ps.r.shape), ps.box)
    _noalloc_twice(L, ps, 2.5, *_oracle(ps, 2.5))


def test_noalloc_rejects_beyond_its_limits():
    E, psm, L = _setup()
    box = (C.c_double * 3)(20.0, 20.0, 20.0)
    # sizes are checked before any device pointer is touched
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 131073, box, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == MD_ERR_CAPACITY
    small = (C.c_double * 3)(6.0, 20.0, 20.0)
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 100, small, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == MD_ERR_UNSUPPORTED
    big = (C.c_double * 3)(200.0, 200.0, 200.0)
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 100, big, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == MD_ERR_CAPACITY  # more cells than MD_NOALLOC_MAX_CELLS
    # axis counts whose product wraps a 64-bit integer: rejected on the first axis
    huge = (C.c_double * 3)(2.5 * 2 ** 22, 2.5 * 2 ** 22, 2.5 * 2 ** 20)
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 131072, huge, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == MD_ERR_CAPACITY
    # a box too large for a 32-bit cell count on one axis
    vast = (C.c_double * 3)(1e300, 20.0, 20.0)
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 100, vast, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == MD_ERR_CAPACITY
