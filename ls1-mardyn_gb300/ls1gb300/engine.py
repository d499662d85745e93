"""ctypes binding of libls1gb300.so and a Python mirror of the reference's
container/integrator interface for this path.

``Engine`` is one ``md_ctx`` (one box).  ``GpuLinkedCells`` and
``GpuLeapfrog`` mirror the method names and call order of the reference's
``ParticleContainer`` (src/particleContainer/ParticleContainer.h:69-296) and
``Integrator``/``Leapfrog`` (src/integrators/Integrator.h:32-84,
src/integrators/Leapfrog.cpp:32-147), so a driver loop reads like
``Simulation::simulateOneTimestep`` (src/Simulation.cpp:1076-1300).

There is no CPU fallback: if the CUDA library is missing the constructor
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import abi
from .phasespace import PhaseSpace

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "libls1gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "ls1gb300.h")
_lib = None

PRECISION = {"fp64": abi.MD_PREC_FP64, "mixed": abi.MD_PREC_MIXED}
PAIR_SCHEME = {"rows": 0, "newton3": 1}


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{abi.ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


def load_library(path: str = LIB_PATH):
    """Load the engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} missing: build it with ls1-mardyn_gb300/build.py")
    L = C.CDLL(path)
    vp, i64, i32, dp, d = C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_double), C.c_double
    L.md_create.argtypes = [C.POINTER(vp), C.POINTER(abi.MdConfig)]
    L.md_destroy.argtypes = [vp]
    L.md_last_error.argtypes = [vp]
    L.md_last_error.restype = C.c_char_p
    L.md_set_components.argtypes = [vp, C.POINTER(abi.MdComponent), i32, dp]
    L.md_upload_molecules.argtypes = [vp, i64, vp, vp, dp, dp, dp, dp]
    L.md_download_molecules.argtypes = [vp, i64] + [vp] * 9
    L.md_set_forces.argtypes = [vp, i64, vp, vp, vp]
    L.md_rebin_and_halo.argtypes = [vp, C.POINTER(abi.MdBinStats)]
    L.md_get_cell_assignment.argtypes = [vp, i64, vp]
    L.md_compute_forces.argtypes = [vp, C.POINTER(abi.MdForcesOut)]
    L.md_integrate_pre.argtypes = [vp, d]
    L.md_integrate_post.argtypes = [vp, d, C.POINTER(abi.MdKineticOut)]
    L.md_run.argtypes = [vp, d, i32, C.POINTER(abi.MdStepRecord)]
    L.md_rmm_forces.argtypes = [vp, d, C.POINTER(abi.MdForcesOut)]
    L.md_rmm_positions.argtypes = [vp, d]
    L.md_rmm_velocities.argtypes = [vp, C.POINTER(abi.MdKineticOut)]
    L.md_rmm_run.argtypes = [vp, d, i32, C.POINTER(abi.MdStepRecord)]
    L.md_sync.argtypes = [vp]
    L.md_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.md_adjoint.argtypes = [vp, d, d, vp, vp, vp, i32]
    L.md_time_kernels.argtypes = [vp, i32, C.POINTER(abi.MdKernelTimes)]
    L.md_rebuilds.argtypes = [vp, C.POINTER(i64)]
    L.md_longrange_homogeneous.argtypes = [vp, i32, dp, dp]
    L.md_set_thermostat.argtypes = [vp, d, i32]
    L.md_apply_thermostat.argtypes = [vp, dp, dp]
    L.md_set_thermostats.argtypes = [vp, vp, i32, dp, i32]
    L.md_thermostat_betas.argtypes = [vp, i32, dp, dp]
    L.md_set_temperature_control.argtypes = [vp, C.POINTER(abi.MdTemperatureControl)]
    L.md_set_simstep.argtypes = [vp, i64]
    L.md_apply_temperature_control.argtypes = [vp, i64]
    L.md_temperature_control_betas.argtypes = [vp, i32, dp, dp]
    L.md_planar_init.argtypes = [vp, C.POINTER(abi.MdPlanarConfig)]
    L.md_planar_apply.argtypes = [vp, dp, dp]
    L.md_write_phasespace_binary.argtypes = [vp, C.c_char_p, d]
    L.md_read_phasespace_binary.argtypes = [vp, C.c_char_p, C.c_char_p, dp, C.POINTER(i64)]
    L.md_batch_create.argtypes = [C.POINTER(vp), C.POINTER(abi.MdBatchConfig)]
    L.md_batch_destroy.argtypes = [vp]
    L.md_batch_last_error.argtypes = [vp]
    L.md_batch_last_error.restype = C.c_char_p
    L.md_batch_upload.argtypes = [vp, vp, vp, dp, dp]
    L.md_batch_compute_forces.argtypes = [vp, C.POINTER(abi.MdBoxSums)]
    L.md_batch_run.argtypes = [vp, d, i32, i32, C.POINTER(abi.MdStepRecord)]
    L.md_batch_download.argtypes = [vp, vp, dp, dp, dp]
    L.md_batch_autotune.argtypes = [vp, d, i32, C.POINTER(abi.MdBatchTuning)]
    L.md_batch_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.md_batch_rebuilds.argtypes = [vp, C.POINTER(i64)]
    _lib = L
    return L


class Engine:
    """One box on the GPU behind the C ABI."""

    def __init__(self, ps: PhaseSpace, rc: float, rc_lj: Optional[float] = None,
                 periodic: Sequence[int] = (1, 1, 1), precision: str = "fp64", skin: float = 0.0,
                 device: int = 0, capacity: int = 0, pair_scheme: str = "rows", arrays=None):
        """pair_scheme "rows": per-molecule candidate rows, each pair evaluated from both sides;
        "newton3": every pair evaluated once (Newton's third law) in mixed precision where the box has
        at least three list cells per periodic axis -- cluster pairs for one component of single-centre
        LJ molecules, half rows with the neighbour's share added by atomics for multi-site molecules --
        rows elsewhere.  arrays: the molecule arrays of ``abi.molecule_arrays(ps)`` to upload (e.g.
        page-locked copies), else made from ps."""
        self.L = load_library()
        self.ps = ps
        self.cfg = abi.make_config(ps.box, rc, rc if rc_lj is None else rc_lj, ps.eps_rf, periodic,
                                   PRECISION[precision], capacity, skin, device,
                                   pair_scheme=PAIR_SCHEME[pair_scheme])
        self.h = C.c_void_p()
        self._check(self.L.md_create(C.byref(self.h), C.byref(self.cfg)), "md_create")
        self.tables = abi.ComponentTables(ps.components, ps.mixing)
        self._check(self.L.md_set_components(self.h, self.tables.array, self.tables.ncomp, self.tables.mixing),
                    "md_set_components")
        self.upload(ps, arrays)

    def _check(self, rc: int, what: str):
        if rc != abi.MD_OK:
            msg = self.L.md_last_error(self.h).decode() if self.h else ""
            raise EngineError(rc, f"{what}: {msg}")

    def upload(self, ps: PhaseSpace, arrays=None):
        ids, comp, r, v, q, Lm = abi.molecule_arrays(ps) if arrays is None else arrays
        self.n = ps.n
        self._check(self.L.md_upload_molecules(self.h, ps.n, ids.ctypes.data, comp.ctypes.data, abi.dptr(r),
                                               abi.dptr(v), abi.dptr(q), abi.dptr(Lm)), "md_upload_molecules")

    def set_forces(self, F: Optional[np.ndarray] = None, M: Optional[np.ndarray] = None,
                   Vi: Optional[np.ndarray] = None):
        """Forces, torques and per-molecule virials (n x 3, upload order) into the state, e.g. after a
        re-upload of edited molecules, whose next pre-force half step kicks with them."""
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (F, M, Vi)]
        self._check(self.L.md_set_forces(self.h, self.n, *(None if a is None else a.ctypes.data for a in arrs)),
                    "md_set_forces")

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.md_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rebin(self) -> abi.MdBinStats:
        st = abi.MdBinStats()
        self._check(self.L.md_rebin_and_halo(self.h, C.byref(st)), "md_rebin_and_halo")
        return st

    def cells(self) -> np.ndarray:
        out = np.zeros(self.n, np.int64)
        self._check(self.L.md_get_cell_assignment(self.h, self.n, out.ctypes.data), "md_get_cell_assignment")
        return out

    def forces(self) -> abi.MdForcesOut:
        fo = abi.MdForcesOut()
        self._check(self.L.md_compute_forces(self.h, C.byref(fo)), "md_compute_forces")
        return fo

    def pre(self, dt: float):
        self._check(self.L.md_integrate_pre(self.h, dt), "md_integrate_pre")

    def post(self, dt: float) -> abi.MdKineticOut:
        ko = abi.MdKineticOut()
        self._check(self.L.md_integrate_post(self.h, dt, C.byref(ko)), "md_integrate_post")
        return ko

    def run(self, dt: float, nsteps: int, record: bool = True) -> Optional[np.ndarray]:
        rec = (abi.MdStepRecord * max(nsteps, 1))() if record else None
        self._check(self.L.md_run(self.h, dt, nsteps, rec), "md_run")
        if not record:
            return None
        return np.array([[x.upot, x.virial, x.summv2, x.sumIw2] for x in rec[:nsteps]])

    # ---- reduced memory mode (LeapfrogRMM + VCP1CLJRMM)
    def rmm_forces(self, dt_inv_m: float) -> abi.MdForcesOut:
        """Force pass that adds dt_inv_m * F to every velocity (no force stored)."""
        out = abi.MdForcesOut()
        self._check(self.L.md_rmm_forces(self.h, dt_inv_m, C.byref(out)), "md_rmm_forces")
        return out

    def rmm_positions(self, dt: float):
        self._check(self.L.md_rmm_positions(self.h, dt), "md_rmm_positions")

    def rmm_velocities(self) -> abi.MdKineticOut:
        out = abi.MdKineticOut()
        self._check(self.L.md_rmm_velocities(self.h, C.byref(out)), "md_rmm_velocities")
        return out

    def rmm_run(self, dt: float, nsteps: int, record: bool = True) -> Optional[np.ndarray]:
        """nsteps LeapfrogRMM steps; rows (Upot, virial, sum v.v, 0)."""
        rec = (abi.MdStepRecord * max(nsteps, 1))() if record else None
        self._check(self.L.md_rmm_run(self.h, dt, nsteps, rec), "md_rmm_run")
        if not record:
            return None
        return np.array([[x.upot, x.virial, x.summv2, x.sumIw2] for x in rec[:nsteps]])

    def sync(self):
        self._check(self.L.md_sync(self.h), "md_sync")

    def stream(self) -> int:
        """cudaStream_t of the context as an integer (for torch.cuda.ExternalStream)."""
        s = C.c_void_p()
        self._check(self.L.md_get_stream(self.h, C.byref(s)), "md_get_stream")
        return s.value or 0

    def rebuilds(self) -> int:
        """List rebuilds since the context was created."""
        c = C.c_int64()
        self._check(self.L.md_rebuilds(self.h, C.byref(c)), "md_rebuilds")
        return c.value

    def time_kernels(self, reps: int = 10) -> abi.MdKernelTimes:
        t = abi.MdKernelTimes()
        self._check(self.L.md_time_kernels(self.h, reps, C.byref(t)), "md_time_kernels")
        return t

    def param_count(self) -> int:
        return sum(2 * len(c.lj) + len(c.charges) + len(c.dipoles) + len(c.quadrupoles) for c in self.ps.components)

    def adjoint(self, gU: float, gW: float, gF: Optional[np.ndarray] = None):
        """(grad_r, grad_params) of gU*Upot + gW*virial (+ sum gF.F) at the
        current state; see md_adjoint in include/ls1gb300.h for the order of
        the parameters."""
        gr = np.zeros((self.n, 3))
        npar = self.param_count()
        gp = np.zeros(max(npar, 1))
        gFa = None if gF is None else np.ascontiguousarray(gF, dtype=np.float64)
        self._check(self.L.md_adjoint(self.h, float(gU), float(gW), None if gFa is None else gFa.ctypes.data,
                                      gr.ctypes.data, gp.ctypes.data, npar), "md_adjoint")
        return gr, gp[:npar]

    def set_thermostat(self, target_temperature: float, explosion_heuristics: bool = True):
        """Global velocity-scaling thermostat at the target (<= 0: NVE), applied by run()."""
        self._check(self.L.md_set_thermostat(self.h, float(target_temperature), int(explosion_heuristics)),
                    "md_set_thermostat")

    def set_thermostats(self, component_thermostat: Sequence[int], targets: Sequence[float],
                        explosion_heuristics: bool = True):
        """Component-wise thermostats: component c on thermostat component_thermostat[c] (ids from 1),
        thermostat t at target targets[t - 1]."""
        m = np.ascontiguousarray(component_thermostat, np.int32)
        t = np.ascontiguousarray(targets, np.float64)
        self._check(self.L.md_set_thermostats(self.h, m.ctypes.data, len(t), abi.dptr(t), int(explosion_heuristics)),
                    "md_set_thermostats")

    def set_temperature_control(self, tc: Optional[dict]):
        """Region-wise temperature control (TemperatureControl with velocity-scaling regions).  ``tc``:
        start, frequency, stop and a list of regions with lower/upper corners (an upper corner None is the
        box length, as the reference's "box"), T, component (1-based, 0 = all), numslabs, exponent,
        directions (bit mask x = 1, y = 2, z = 4) and an optional ramp (start, end, update_start,
        update_stop, update_freq).  A region with method "andersen" takes nu instead of numslabs, exponent,
        directions and ramp; ``tc`` then also gives timestep and seed.  None switches it off."""
        if tc is None:
            self._check(self.L.md_set_temperature_control(self.h, None), "md_set_temperature_control")
            return
        c = abi.MdTemperatureControl()
        c.start, c.frequency, c.stop = int(tc["start"]), int(tc["frequency"]), int(tc["stop"])
        c.nregions = len(tc["regions"])
        c.timestep, c.seed = float(tc.get("timestep", 0.0)), int(tc.get("seed", 8624))
        for k, r in enumerate(tc["regions"]):
            g = c.regions[k]
            for d in range(3):
                g.lower[d] = float(r["lower"][d])
                g.upper[d] = float(self.ps.box[d] if r["upper"][d] is None else r["upper"][d])
            g.target_temperature = float(r["T"])
            g.component = int(r["component"])
            if r.get("method", "velocity_scaling") == "andersen":
                g.method, g.nu = 1, float(r["nu"])
                continue
            g.numslabs = int(r["numslabs"])
            g.exponent, g.directions = float(r["exponent"]), int(r["directions"])
            ramp = r.get("ramp")
            g.ramp_enabled = 1 if ramp else 0
            if ramp:
                g.ramp_start, g.ramp_end = float(ramp["start"]), float(ramp["end"])
                g.ramp_update_start, g.ramp_update_stop = int(ramp["update_start"]), int(ramp["update_stop"])
                g.ramp_update_freq = int(ramp["update_freq"])
        self._check(self.L.md_set_temperature_control(self.h, C.byref(c)), "md_set_temperature_control")

    def apply_temperature_control(self, step: int):
        """The temperature control of step ``step`` (after md_integrate_post)."""
        self._check(self.L.md_apply_temperature_control(self.h, int(step)), "md_apply_temperature_control")

    def set_simstep(self, step: int):
        self._check(self.L.md_set_simstep(self.h, int(step)), "md_set_simstep")

    def temperature_control_betas(self, region: int, numslabs: int):
        bt, br = np.zeros(numslabs), np.zeros(numslabs)
        self._check(self.L.md_temperature_control_betas(self.h, int(region), abi.dptr(bt), abi.dptr(br)),
                    "md_temperature_control_betas")
        return bt, br

    def thermostat_betas(self, thermostat: int = 0):
        bt, br = C.c_double(), C.c_double()
        self._check(self.L.md_thermostat_betas(self.h, int(thermostat), C.byref(bt), C.byref(br)),
                    "md_thermostat_betas")
        return bt.value, br.value

    def apply_thermostat(self):
        """One thermostat application after post(); returns (beta_trans, beta_rot)."""
        bt, br = C.c_double(), C.c_double()
        self._check(self.L.md_apply_thermostat(self.h, C.byref(bt), C.byref(br)), "md_apply_thermostat")
        return bt.value, br.value

    def longrange_homogeneous(self, add_to_molecule_virial: bool = False):
        """(UpotCorr, VirialCorr) of the homogeneous long-range correction."""
        u, w = C.c_double(), C.c_double()
        self._check(self.L.md_longrange_homogeneous(self.h, int(add_to_molecule_virial), C.byref(u), C.byref(w)),
                    "md_longrange_homogeneous")
        return u.value, w.value

    def planar_init(self, slabs: int, frequency: int = 10, region: Optional[Sequence[float]] = None,
                    target_temperature: Optional[float] = None):
        """Planar long-range correction (longRange/Planar): slabs along y, profiles every `frequency` calls,
        force corrections in the y range `region` (default: the whole box)."""
        lo, hi = (0.0, float(self.ps.box[1])) if region is None else region
        T = float(self.ps.temperature) if target_temperature is None else target_temperature
        cfg = abi.MdPlanarConfig(int(slabs), int(frequency), float(lo), float(hi), T)
        self._check(self.L.md_planar_init(self.h, C.byref(cfg)), "md_planar_init")

    def planar_apply(self):
        """(UpotCorr, VirialCorr) of this call; adds the corrections to F, M and Vi."""
        u, w = C.c_double(), C.c_double()
        self._check(self.L.md_planar_apply(self.h, C.byref(u), C.byref(w)), "md_planar_apply")
        return u.value, w.value

    def write_phasespace_binary(self, prefix: str, time: float = 0.0):
        """<prefix>.header.xml + <prefix>.dat in ls1's binary checkpoint format."""
        self._check(self.L.md_write_phasespace_binary(self.h, os.fsencode(prefix), time), "md_write_phasespace_binary")

    def read_phasespace_binary(self, header: str, data: str):
        """Replace the molecules by those of a binary phase-space file pair; returns (time, n)."""
        t, n = C.c_double(), C.c_int64()
        self._check(self.L.md_read_phasespace_binary(self.h, os.fsencode(header), os.fsencode(data), C.byref(t),
                                                     C.byref(n)), "md_read_phasespace_binary")
        self.n = n.value
        return t.value, n.value

    def write_checkpoint(self, prefix: str, step: int, time: float, num_steps: int = 0, write_frequency: int = 1,
                         incremental: bool = True) -> str:
        """CheckpointWriter::endStep with the binary type (src/io/CheckpointWriter.cpp:56-80):
        <prefix>[-<step / frequency, zero-padded>].restart{.header.xml,.dat}; returns the name."""
        name = prefix
        if incremental:
            digits = int(np.ceil(np.log(float(num_steps // write_frequency)) / np.log(10.0))) if num_steps else 0
            name += "-" + str(step // write_frequency).rjust(max(digits, 0), "0")
        name += ".restart"
        self.write_phasespace_binary(name, time)
        return name

    def molecules(self, out: Optional[dict] = None) -> dict:
        """All molecules in upload order; `out` (same keys, e.g. page-locked arrays from pinned.empty) receives
        them instead of new arrays."""
        n = self.n
        if out is None:
            out = dict(ids=np.zeros(n, np.uint64), comp=np.zeros(n, np.int32), r=np.zeros((n, 3)),
                       v=np.zeros((n, 3)), q=np.zeros((n, 4)), L=np.zeros((n, 3)), F=np.zeros((n, 3)),
                       M=np.zeros((n, 3)), Vi=np.zeros((n, 3)))
        self._check(self.L.md_download_molecules(self.h, n, *(out[k].ctypes.data for k in
                                                              ("ids", "comp", "r", "v", "q", "L", "F", "M", "Vi"))),
                    "md_download_molecules")
        return out


class GpuLinkedCells:
    """Mirror of the reference's ParticleContainer calls used on this path."""

    def __init__(self, ps: PhaseSpace, cutoff: float, lj_cutoff: Optional[float] = None, **kw):
        self.engine = Engine(ps, cutoff, lj_cutoff, **kw)
        self._cutoff = cutoff

    # ParticleContainer::update + DomainDecompBase::exchangeMolecules + updateMoleculeCaches
    def update(self) -> abi.MdBinStats:
        return self.engine.rebin()

    # ParticleContainer::traverseCells(VectorizedCellProcessor&) + Simulation::updateForces
    def traverseCells(self) -> abi.MdForcesOut:
        return self.engine.forces()

    def getNumberOfParticles(self) -> int:
        return self.engine.n

    def getCutoff(self) -> float:
        return self._cutoff

    def getCellIndexOfMolecules(self) -> np.ndarray:
        return self.engine.cells()

    def molecules(self) -> dict:
        return self.engine.molecules()


class GpuLeapfrog:
    """Mirror of Leapfrog's state machine (Leapfrog.cpp:32-147)."""

    def __init__(self, dt: float):
        self.dt = dt

    def eventNewTimestep(self, cells: GpuLinkedCells):
        cells.engine.pre(self.dt)

    def eventForcesCalculated(self, cells: GpuLinkedCells) -> abi.MdKineticOut:
        return cells.engine.post(self.dt)


class GpuLeapfrogRMM:
    """Mirror of LeapfrogRMM with its cell processors (LeapfrogRMM.cpp:42-107,
    VCP1CLJRMM.cpp:41-44, Simulation.cpp:902-938): prepare() is the initial
    force pass with the half kick dt/(2m), then per step eventNewTimestep
    (positions), traverseCells (forces with the kick dt/m) and
    eventForcesCalculated (N, sum v.v)."""

    def __init__(self, dt: float, mass: float):
        self.dt = dt
        self.dt_inv_m = dt / mass

    def prepare(self, cells: GpuLinkedCells) -> abi.MdForcesOut:
        return cells.engine.rmm_forces(self.dt_inv_m * 0.5)

    def eventNewTimestep(self, cells: GpuLinkedCells):
        cells.engine.rmm_positions(self.dt)

    def traverseCells(self, cells: GpuLinkedCells) -> abi.MdForcesOut:
        return cells.engine.rmm_forces(self.dt_inv_m)

    def eventForcesCalculated(self, cells: GpuLinkedCells) -> abi.MdKineticOut:
        return cells.engine.rmm_velocities()
