"""The allocation-free entry point md_forces_lj_noalloc, for callers that
cannot allocate device memory (graphs owned by a larger application, pooled
device memory, real-time drivers): called twice in a row through the C ABI
on device buffers the caller owns, it must reproduce the forces, Upot and
virial of the regular entry point (md_compute_forces, FP64) to 1e-10
relative; oversize requests are rejected before any device work.
This file is collected last on purpose."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))

pytestmark = pytest.mark.gpu


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


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    E, psm, L = _setup()
    ps = psm.lj_fcc(8, 0.8, 1.0, seed=13)
    ps.r = ps.r + np.random.default_rng(13).uniform(-0.12, 0.12, ps.r.shape)
    ps.r = np.mod(ps.r, ps.box)
    rc = 2.5
    e = E.Engine(ps, rc, precision="fp64")
    fo = e.forces()
    F_ref = e.molecules()["F"]
    e.close()
    r = torch.tensor(ps.r, dtype=torch.float64, device="cuda")
    F = torch.empty_like(r)
    uv = torch.empty(2, dtype=torch.float64, device="cuda")
    box = (C.c_double * 3)(*ps.box)
    for _ in range(2):
        F.fill_(float("nan"))
        uv.fill_(float("nan"))
        torch.cuda.synchronize()
        rc_ = L.md_forces_lj_noalloc(r.data_ptr(), ps.n, box, rc, 1.0, 1.0, 0.0, F.data_ptr(), uv.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc_ == 0
        Fn = F.cpu().numpy()
        assert np.abs(Fn - F_ref).max() <= 1e-10 * np.abs(F_ref).max()
        u, w = uv.cpu().numpy()
        assert abs(u - fo.upot) <= 1e-10 * abs(fo.upot)
        assert abs(w - fo.virial) <= 1e-10 * abs(fo.virial)


def test_noalloc_rejects_beyond_its_limits():
    E, psm, L = _setup()
    box = (C.c_double * 3)(20.0, 20.0, 20.0)
    # sizes are checked before any device pointer is touched
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 131073, box, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == 3   # MD_ERR_CAPACITY
    small = (C.c_double * 3)(6.0, 20.0, 20.0)
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 100, small, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == 6   # MD_ERR_UNSUPPORTED
    big = (C.c_double * 3)(200.0, 200.0, 200.0)
    assert L.md_forces_lj_noalloc(C.c_void_p(16), 100, big, 2.5, 1.0, 1.0, 0.0, C.c_void_p(16),
                                  C.c_void_p(16), None) == 3   # more cells than MD_NOALLOC_MAX_CELLS
