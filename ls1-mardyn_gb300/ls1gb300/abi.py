"""ctypes mirror of include/ls1gb300.h and helpers that turn a PhaseSpace into
the plain structs the C ABI takes.

The structs here are byte-for-byte the ones declared in include/ls1gb300.h;
``test_abi`` checks their sizes against the compiled library.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from .phasespace import Component, PhaseSpace

MD_OK = 0
MD_ERR_ARG = 1
MD_ERR_CUDA = 2
MD_ERR_CAPACITY = 3
MD_ERR_STATE = 4
MD_ERR_DEVICE = 5
MD_ERR_UNSUPPORTED = 6
MD_PREC_FP64 = 0
MD_PREC_MIXED = 1
MD_NUM_KINDS = 7
KIND_NAMES = ("LJ", "C-C", "C-D", "D-D", "C-Q", "D-Q", "Q-Q")

ERROR_NAMES = {MD_ERR_ARG: "MD_ERR_ARG", MD_ERR_CUDA: "MD_ERR_CUDA", MD_ERR_CAPACITY: "MD_ERR_CAPACITY",
               MD_ERR_STATE: "MD_ERR_STATE", MD_ERR_DEVICE: "MD_ERR_DEVICE",
               MD_ERR_UNSUPPORTED: "MD_ERR_UNSUPPORTED"}


class MdConfig(C.Structure):
    _fields_ = [("box_min", C.c_double * 3), ("box_max", C.c_double * 3), ("rc", C.c_double),
                ("rc_lj", C.c_double), ("eps_rf", C.c_double), ("periodic", C.c_int32 * 3),
                ("precision", C.c_int32), ("capacity", C.c_int64), ("skin", C.c_double),
                ("device", C.c_int32), ("pair_scheme", C.c_int32)]


class MdComponent(C.Structure):
    _fields_ = [("n_lj", C.c_int32), ("n_charge", C.c_int32), ("n_dipole", C.c_int32),
                ("n_quadrupole", C.c_int32), ("lj", C.POINTER(C.c_double)), ("charge", C.POINTER(C.c_double)),
                ("dipole", C.POINTER(C.c_double)), ("quadrupole", C.POINTER(C.c_double)),
                ("inertia", C.c_double * 3)]


class MdBinStats(C.Structure):
    _fields_ = [("n_inner", C.c_int64), ("n_halo", C.c_int64), ("max_occupancy", C.c_int64),
                ("n_wrapped", C.c_int64), ("cells", C.c_int32 * 3), ("reserved", C.c_int32),
                ("cell_length", C.c_double * 3)]


class MdForcesOut(C.Structure):
    _fields_ = [("upot", C.c_double), ("virial", C.c_double), ("my_rf", C.c_double), ("upot6lj", C.c_double),
                ("upot_xpoles", C.c_double), ("virial_pairs", C.c_double), ("mol_pairs", C.c_int64),
                ("site_pairs", C.c_int64 * MD_NUM_KINDS)]


class MdKineticOut(C.Structure):
    _fields_ = [("summv2", C.c_double), ("sumIw2", C.c_double), ("n", C.c_int64), ("rot_dof", C.c_int64)]


class MdPlanarConfig(C.Structure):
    _fields_ = [("slabs", C.c_int32), ("frequency", C.c_int32), ("region_lo", C.c_double), ("region_hi", C.c_double),
                ("target_temperature", C.c_double)]


MD_TC_MAX_REGIONS = 8
MD_TC_MAX_SLABS = 64


class MdTcRegion(C.Structure):
    _fields_ = [("lower", C.c_double * 3), ("upper", C.c_double * 3), ("target_temperature", C.c_double),
                ("component", C.c_int32), ("numslabs", C.c_int32), ("exponent", C.c_double),
                ("directions", C.c_int32), ("ramp_enabled", C.c_int32), ("ramp_start", C.c_double),
                ("ramp_end", C.c_double), ("ramp_update_start", C.c_int64), ("ramp_update_stop", C.c_int64),
                ("ramp_update_freq", C.c_int64), ("method", C.c_int32), ("reserved", C.c_int32), ("nu", C.c_double)]


class MdTemperatureControl(C.Structure):
    _fields_ = [("start", C.c_int64), ("frequency", C.c_int64), ("stop", C.c_int64), ("nregions", C.c_int32),
                ("reserved", C.c_int32), ("regions", MdTcRegion * MD_TC_MAX_REGIONS), ("timestep", C.c_double),
                ("seed", C.c_uint64)]


class MdStepRecord(C.Structure):
    _fields_ = [("upot", C.c_double), ("virial", C.c_double), ("summv2", C.c_double), ("sumIw2", C.c_double)]


class MdKernelTimes(C.Structure):
    _fields_ = [("force_ms", C.c_double), ("pre_ms", C.c_double), ("post_ms", C.c_double),
                ("rebuild_ms", C.c_double), ("mean_candidates", C.c_double), ("rebuilds", C.c_int64),
                ("launches_per_step", C.c_int32), ("launches_per_rebuild", C.c_int32),
                ("adjoint_ms", C.c_double), ("step_force_ms", C.c_double), ("lf_ms", C.c_double),
                ("pair_scheme", C.c_int32), ("cluster_size", C.c_int32)]


class MdBatchConfig(C.Structure):
    _fields_ = [("nbox", C.c_int32), ("precision", C.c_int32), ("box_len", C.POINTER(C.c_double)),
                ("rc", C.c_double), ("epsilon", C.c_double), ("sigma", C.c_double), ("mass", C.c_double),
                ("shifted", C.c_int32), ("threads_per_molecule", C.c_int32), ("skin", C.c_double),
                ("device", C.c_int32), ("reserved", C.c_int32), ("cell_occupancy", C.c_double)]


class MdBoxSums(C.Structure):
    _fields_ = [("upot", C.c_double), ("virial", C.c_double), ("pairs", C.c_int64)]


MD_BATCH_TUNE_MAX = 16


class MdBatchTuning(C.Structure):
    _fields_ = [("skin", C.c_double), ("threads_per_molecule", C.c_int32), ("ntrials", C.c_int32),
                ("ms_per_step", C.c_double), ("trial_skin", C.c_double * MD_BATCH_TUNE_MAX),
                ("trial_tpm", C.c_int32 * MD_BATCH_TUNE_MAX), ("trial_ms_per_step", C.c_double * MD_BATCH_TUNE_MAX),
                ("cell_occupancy", C.c_double), ("trial_occupancy", C.c_double * MD_BATCH_TUNE_MAX)]


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_config(box, rc: float, rc_lj: float, eps_rf: float, periodic: Sequence[int] = (1, 1, 1),
                precision: int = MD_PREC_FP64, capacity: int = 0, skin: float = 0.0, device: int = 0,
                box_min=(0.0, 0.0, 0.0), pair_scheme: int = 0) -> MdConfig:
    cfg = MdConfig()
    for d in range(3):
        cfg.box_min[d] = float(box_min[d])
        cfg.box_max[d] = float(box_min[d]) + float(box[d])
        cfg.periodic[d] = int(periodic[d])
    cfg.rc, cfg.rc_lj, cfg.eps_rf = float(rc), float(rc_lj), float(eps_rf)
    cfg.precision, cfg.capacity, cfg.skin, cfg.device = int(precision), int(capacity), float(skin), int(device)
    cfg.pair_scheme = int(pair_scheme)
    return cfg


class ComponentTables:
    """md_component array plus the numpy buffers it points into."""

    def __init__(self, comps: List[Component], mixing: Sequence[Sequence[float]]):
        self._keep = []
        self.array = (MdComponent * len(comps))()
        for k, c in enumerate(comps):
            lj = np.array([[*s.r, s.m, s.eps, s.sigma, s.shift6] for s in c.lj], dtype=np.float64).reshape(-1, 7)
            ch = np.array([[*s.r, s.m, s.q] for s in c.charges], dtype=np.float64).reshape(-1, 5)
            di = np.array([[*s.r, *s.e, s.abs] for s in c.dipoles], dtype=np.float64).reshape(-1, 7)
            qu = np.array([[*s.r, *s.e, s.abs] for s in c.quadrupoles], dtype=np.float64).reshape(-1, 7)
            bufs = [np.ascontiguousarray(x) for x in (lj, ch, di, qu)]
            self._keep.extend(bufs)
            m = self.array[k]
            m.n_lj, m.n_charge, m.n_dipole, m.n_quadrupole = (b.shape[0] for b in bufs)
            m.lj, m.charge, m.dipole, m.quadrupole = (dptr(b) for b in bufs)
            for d in range(3):
                m.inertia[d] = float(c.I_override[d])
        self.ncomp = len(comps)
        mix = np.ascontiguousarray(np.array(mixing, dtype=np.float64).reshape(-1, 2))
        if mix.shape[0] < self.ncomp * (self.ncomp - 1) // 2:
            mix = np.ones((self.ncomp * (self.ncomp - 1) // 2, 2))
        self._keep.append(mix)
        self.mixing = dptr(mix)


def molecule_arrays(ps: PhaseSpace):
    """Contiguous copies of the per-molecule state in the ABI's layout."""
    return (np.ascontiguousarray(ps.ids, dtype=np.uint64), np.ascontiguousarray(ps.comp, dtype=np.int32),
            np.ascontiguousarray(ps.r, dtype=np.float64), np.ascontiguousarray(ps.v, dtype=np.float64),
            np.ascontiguousarray(ps.q, dtype=np.float64), np.ascontiguousarray(ps.L, dtype=np.float64))
