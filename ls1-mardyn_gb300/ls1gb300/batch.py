"""Batches of independent periodic 1CLJ boxes on one GPU (``md_batch_*`` of
the C ABI) and the seeded generator of such batches.

``Batch`` owns one ``md_batch``: all boxes advance together, every kernel
launch covers all boxes, and a run is captured as CUDA graphs of
``graph_steps`` steps.  Per-box Upot, virial and sum m v^2 come back for every
step.  There is no CPU path: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import abi
from .engine import PRECISION, EngineError, load_library
from .phasespace import PhaseSpace, fcc_positions, maxwell_boltzmann, one_center_lj


@dataclass
class Box:
    """One periodic box: edge lengths, positions and velocities (n x 3)."""
    L: np.ndarray
    r: np.ndarray
    v: np.ndarray
    rho: float = 0.0
    T: float = 0.0

    @property
    def n(self) -> int:
        return self.r.shape[0]

    def to_phasespace(self, shifted: bool = False, rc: float = 2.5) -> PhaseSpace:
        """The box as a one-box phase space (eps = sigma = m = 1), ids 1..n."""
        n = self.n
        q = np.zeros((n, 4)); q[:, 0] = 1.0
        return PhaseSpace(np.array(self.L, dtype=np.float64), [one_center_lj(shifted=shifted, rc=rc)], [], 1.0e10,
                          np.arange(1, n + 1, dtype=np.uint64), np.zeros(n, np.int32), self.r.copy(), self.v.copy(),
                          q, np.zeros((n, 3)), self.T)


def random_boxes(nbox: int, n_min: int, n_max: int, rho_range=(0.05, 0.85), t_range=(0.7, 1.3),
                 seed: int = 0, mass: float = 1.0) -> List[Box]:
    """Seeded batch of cubic 1CLJ boxes: N log-uniform in [n_min, n_max],
    rho* and T* uniform in the given ranges.  Molecules take N random sites of
    the smallest fcc lattice with at least N sites that fills the box; velocities
    are Maxwell-Boltzmann at T* with the net momentum removed."""
    rng = np.random.default_rng(seed)
    boxes = []
    for _ in range(nbox):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        rho = float(rng.uniform(*rho_range))
        T = float(rng.uniform(*t_range))
        L = (n / rho) ** (1.0 / 3.0)
        m = int(np.ceil((n / 4.0) ** (1.0 / 3.0) - 1e-9))
        sites = fcc_positions((m, m, m), L / m)
        pick = np.sort(rng.choice(sites.shape[0], size=n, replace=False))
        r = sites[pick]
        v = maxwell_boltzmann(rng, n, np.full(n, mass), T)
        boxes.append(Box(L=np.array([L, L, L]), r=np.ascontiguousarray(r), v=np.ascontiguousarray(v), rho=rho, T=T))
    return boxes


class Batch:
    """Many boxes on one GPU behind the md_batch C ABI."""

    def __init__(self, boxes: Sequence[Box], rc: float, precision: str = "mixed", skin: float = -1.0,
                 threads_per_molecule: int = 0, epsilon: float = 1.0, sigma: float = 1.0, mass: float = 1.0,
                 shifted: bool = False, device: int = 0, cell_occupancy: float = 0.0):
        self.L = load_library()
        self.h = C.c_void_p()
        self.nbox = len(boxes)
        self._len = np.ascontiguousarray(np.array([b.L for b in boxes], dtype=np.float64).reshape(-1))
        cfg = abi.MdBatchConfig()
        cfg.nbox = self.nbox
        cfg.precision = PRECISION[precision]
        cfg.box_len = self._len.ctypes.data_as(C.POINTER(C.c_double))
        cfg.rc = rc
        cfg.epsilon, cfg.sigma, cfg.mass = epsilon, sigma, mass
        cfg.shifted = int(shifted)
        cfg.threads_per_molecule = threads_per_molecule
        cfg.skin = skin
        cfg.device = device
        cfg.cell_occupancy = cell_occupancy
        rc_ = self.L.md_batch_create(C.byref(self.h), C.byref(cfg))
        if rc_ != abi.MD_OK:
            msg = self.L.md_batch_last_error(self.h).decode() if self.h.value else ""
            self.close()
            raise EngineError(rc_, f"md_batch_create: {msg}")
        self.upload(boxes)

    def _check(self, rc: int, what: str):
        if rc != abi.MD_OK:
            raise EngineError(rc, f"{what}: {self.L.md_batch_last_error(self.h).decode()}")

    def upload(self, boxes: Sequence[Box]):
        counts = np.array([b.n for b in boxes], dtype=np.int64)
        self.box_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.n = int(self.box_start[-1])
        r = np.ascontiguousarray(np.concatenate([b.r for b in boxes]), dtype=np.float64)
        v = np.ascontiguousarray(np.concatenate([b.v for b in boxes]), dtype=np.float64)
        ids = np.arange(1, self.n + 1, dtype=np.uint64)
        self._check(self.L.md_batch_upload(self.h, self.box_start.ctypes.data, ids.ctypes.data, abi.dptr(r),
                                           abi.dptr(v)), "md_batch_upload")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.md_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forces(self) -> np.ndarray:
        """Per-box (Upot, virial, pairs) at the current positions."""
        out = (abi.MdBoxSums * self.nbox)()
        self._check(self.L.md_batch_compute_forces(self.h, out), "md_batch_compute_forces")
        return np.array([(o.upot, o.virial, o.pairs) for o in out])

    def run(self, dt: float, nsteps: int, graph_steps: int = 100, record: bool = True) -> Optional[np.ndarray]:
        """nsteps NVE steps; returns (nsteps, nbox, 4): Upot, virial, sum m v^2, 0."""
        rec = (abi.MdStepRecord * max(1, nsteps * self.nbox))() if record else None
        self._check(self.L.md_batch_run(self.h, dt, nsteps, graph_steps, rec), "md_batch_run")
        if not record:
            return None
        a = np.frombuffer(rec, dtype=np.float64).reshape(-1, 4)[: nsteps * self.nbox]
        return a.reshape(nsteps, self.nbox, 4).copy()

    def molecules(self):
        ids = np.zeros(self.n, dtype=np.uint64)
        r, v, F = (np.zeros((self.n, 3)) for _ in range(3))
        self._check(self.L.md_batch_download(self.h, ids.ctypes.data, abi.dptr(r), abi.dptr(v), abi.dptr(F)),
                    "md_batch_download")
        return {"ids": ids, "r": r, "v": v, "F": F}

    def autotune(self, dt: float, trial_steps: int = 30) -> dict:
        t = abi.MdBatchTuning()
        self._check(self.L.md_batch_autotune(self.h, dt, trial_steps, C.byref(t)), "md_batch_autotune")
        trials = [(t.trial_skin[k], t.trial_tpm[k], t.trial_occupancy[k], t.trial_ms_per_step[k])
                  for k in range(t.ntrials)]
        return {"skin": t.skin, "threads_per_molecule": t.threads_per_molecule, "cell_occupancy": t.cell_occupancy,
                "ms_per_step": t.ms_per_step, "trials": trials}

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.L.md_batch_get_stream(self.h, C.byref(s)), "md_batch_get_stream")
        return s.value or 0

    def rebuilds(self) -> int:
        c = C.c_int64()
        self._check(self.L.md_batch_rebuilds(self.h, C.byref(c)), "md_batch_rebuilds")
        return int(c.value)
