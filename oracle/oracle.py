"""ctypes binding of the C oracle, plus the numpy restatement of the
Andersen regions of TemperatureControl (test infrastructure only).

Used as the checker by tests/, by ``__graft_entry__.smoke()`` and by the CPU
baseline of ``bench.py``; the engine never imports it.  ``build()`` compiles
``liboracle.so`` with the Makefile beside this file.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if os.path.join(ROOT, "ls1-mardyn_gb300") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
from ls1gb300 import abi  # noqa: E402

LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "md_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i64, i32, dp = C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(abi.MdConfig), C.POINTER(abi.MdComponent), i32, dp]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [i32]
        L.orc_set_molecules.argtypes = [vp, i64, C.c_void_p, C.c_void_p, dp, dp, dp, dp]
        L.orc_num_molecules.restype = i64
        L.orc_num_molecules.argtypes = [vp]
        L.orc_get_molecules.argtypes = [vp, i64] + [C.c_void_p] * 9
        L.orc_rebin_and_halo.argtypes = [vp, C.POINTER(abi.MdBinStats)]
        L.orc_get_cells.argtypes = [vp, i64, C.c_void_p]
        L.orc_forces.argtypes = [vp, C.POINTER(abi.MdForcesOut), dp]
        L.orc_pre.argtypes = [vp, C.c_double]
        L.orc_post.argtypes = [vp, C.c_double, C.POINTER(abi.MdKineticOut)]
        L.orc_run.argtypes = [vp, C.c_double, i32, C.POINTER(abi.MdStepRecord)]
        L.orc_rmm_forces.argtypes = [vp, C.c_double, C.POINTER(abi.MdForcesOut)]
        L.orc_rmm_positions.argtypes = [vp, C.c_double]
        L.orc_rmm_velocities.argtypes = [vp, C.POINTER(abi.MdKineticOut)]
        L.orc_rmm_run.argtypes = [vp, C.c_double, i32, C.POINTER(abi.MdStepRecord)]
        L.orc_longrange_homogeneous.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_set_thermostat.argtypes = [vp, C.c_double, i32]
        _lib = L
    return _lib


class Oracle:
    """One box held by the CPU oracle (same call sequence as the engine)."""

    def __init__(self, ps, rc, rc_lj=None, periodic=(1, 1, 1), threads: int = 1):
        L = lib()
        self.ps = ps
        self.cfg = abi.make_config(ps.box, rc, rc if rc_lj is None else rc_lj, ps.eps_rf, periodic)
        self.tables = abi.ComponentTables(ps.components, ps.mixing)
        L.orc_set_threads(threads)
        self.h = L.orc_create(C.byref(self.cfg), self.tables.array, self.tables.ncomp, self.tables.mixing)
        if not self.h:
            raise RuntimeError("orc_create failed")
        ids, comp, r, v, q, Lm = abi.molecule_arrays(ps)
        rc_ = L.orc_set_molecules(self.h, ps.n, ids.ctypes.data, comp.ctypes.data, abi.dptr(r), abi.dptr(v),
                                  abi.dptr(q), abi.dptr(Lm))
        if rc_:
            raise RuntimeError(f"orc_set_molecules: {rc_}")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def n(self) -> int:
        return int(lib().orc_num_molecules(self.h))

    def rebin(self):
        st = abi.MdBinStats()
        rc = lib().orc_rebin_and_halo(self.h, C.byref(st))
        if rc:
            raise RuntimeError(f"orc_rebin_and_halo: {rc}")
        return st

    def cells(self) -> np.ndarray:
        out = np.zeros(self.n, np.int64)
        lib().orc_get_cells(self.h, self.n, out.ctypes.data)
        return out

    def forces(self):
        fo = abi.MdForcesOut()
        kc = np.zeros(8)
        lib().orc_forces(self.h, C.byref(fo), abi.dptr(kc))
        return fo, kc

    def pre(self, dt):
        lib().orc_pre(self.h, dt)

    def post(self, dt):
        ko = abi.MdKineticOut()
        lib().orc_post(self.h, dt, C.byref(ko))
        return ko

    def set_thermostat(self, target_temperature, explosion_heuristics=True):
        lib().orc_set_thermostat(self.h, target_temperature, int(explosion_heuristics))

    def longrange_homogeneous(self):
        """(UpotCorr, VirialCorr) of the homogeneous long-range correction."""
        u, w = C.c_double(), C.c_double()
        rc = lib().orc_longrange_homogeneous(self.h, C.byref(u), C.byref(w))
        if rc:
            raise RuntimeError(f"orc_longrange_homogeneous: {rc}")
        return u.value, w.value

    def run(self, dt, nsteps):
        rec = (abi.MdStepRecord * max(nsteps, 1))()
        rc = lib().orc_run(self.h, dt, nsteps, rec)
        if rc:
            raise RuntimeError(f"orc_run: {rc}")
        return np.array([[x.upot, x.virial, x.summv2, x.sumIw2] for x in rec[:nsteps]])

    def rmm_forces(self, dt_inv_m):
        """Reduced memory mode force pass: forces, then v += dt_inv_m F."""
        fo = abi.MdForcesOut()
        rc = lib().orc_rmm_forces(self.h, dt_inv_m, C.byref(fo))
        if rc:
            raise RuntimeError(f"orc_rmm_forces: {rc}")
        return fo

    def rmm_positions(self, dt):
        lib().orc_rmm_positions(self.h, dt)

    def rmm_velocities(self):
        ko = abi.MdKineticOut()
        lib().orc_rmm_velocities(self.h, C.byref(ko))
        return ko

    def rmm_run(self, dt, nsteps):
        rec = (abi.MdStepRecord * max(nsteps, 1))()
        rc = lib().orc_rmm_run(self.h, dt, nsteps, rec)
        if rc:
            raise RuntimeError(f"orc_rmm_run: {rc}")
        return np.array([[x.upot, x.virial, x.summv2, x.sumIw2] for x in rec[:nsteps]])

    def molecules(self):
        n = self.n
        out = dict(ids=np.zeros(n, np.uint64), comp=np.zeros(n, np.int32), r=np.zeros((n, 3)), v=np.zeros((n, 3)),
                   q=np.zeros((n, 4)), L=np.zeros((n, 3)), F=np.zeros((n, 3)), M=np.zeros((n, 3)),
                   Vi=np.zeros((n, 3)))
        lib().orc_get_molecules(self.h, n, *(out[k].ctypes.data for k in
                                             ("ids", "comp", "r", "v", "q", "L", "F", "M", "Vi")))
        return out


# ---------------------------------------------------------------- binary phase space
# ls1's binary checkpoint format, restated with numpy (test infrastructure:
# the checker of the engine's device-side writer and reader).
#   record (FullMolecule::writeBinary, src/molecules/FullMolecule.cpp:448-470):
#     id u64, component u32 (1-based), r[3], v[3], q[4] (w, x, y, z), L[3]
#     as little-endian doubles, 116 bytes packed;
#   formats read by BinaryReader::readPhaseSpace (src/io/BinaryReader.cpp:186-226):
#     ICRVQD as above, ICRV (no q, L: q = (1, 0, 0, 0), L = 0), IRV (no
#     component either: component 1);
#   header (Domain::writeCheckpointHeaderXML, src/Domain.cpp:581-605):
#     <time>, <length>/<x|y|z> in "%21.15e", <number>, <format type="...">.
RECORD_DTYPES = {
    "ICRVQD": np.dtype([("id", "<u8"), ("cid", "<u4"), ("r", "<f8", 3), ("v", "<f8", 3), ("q", "<f8", 4),
                        ("L", "<f8", 3)]),
    "ICRV": np.dtype([("id", "<u8"), ("cid", "<u4"), ("r", "<f8", 3), ("v", "<f8", 3)]),
    "IRV": np.dtype([("id", "<u8"), ("r", "<f8", 3), ("v", "<f8", 3)]),
}


def phasespace_binary_records(ids, comp, r, v, q, L) -> bytes:
    """ICRVQD records of the given molecules in the given order (comp 0-based)."""
    a = np.zeros(len(ids), RECORD_DTYPES["ICRVQD"])
    a["id"] = ids
    a["cid"] = np.asarray(comp) + 1
    a["r"], a["v"], a["q"], a["L"] = r, v, q, L
    return a.tobytes()


def phasespace_binary_header(box, n, time) -> str:
    """The header text Domain::writeCheckpointHeaderXML writes for one process."""
    f = lambda x: "%21.15e" % x  # noqa: E731
    return ("<?xml version='1.0' encoding='UTF-8'?>\n<mardyn version=\"20100525\" >\n\t<headerinfo>\n"
            f"\t\t<time>{f(time)}</time>\n\t\t<length>\n"
            f"\t\t\t<x>{f(box[0])}</x> <y>{f(box[1])}</y> <z>{f(box[2])}</z>\n\t\t</length>\n"
            f"\t\t<number>{int(n)}</number>\n\t\t<format type=\"ICRVQD\"/>\n\t</headerinfo>\n</mardyn>\n")


def read_phasespace_binary(header_text: str, data: bytes):
    """(time, box, dict of arrays in file order, comp 0-based) of a header and data pair."""
    import re
    get = lambda tag: re.search(r"<%s>\s*([^<]+?)\s*</%s>" % (tag, tag), header_text).group(1)  # noqa: E731
    time = float(get("time"))
    box = np.array([float(get("x")), float(get("y")), float(get("z"))])
    n = int(get("number"))
    fmt = re.search(r"<format\s+type=\"([A-Z]+)\"", header_text).group(1)
    a = np.frombuffer(data, RECORD_DTYPES[fmt], count=n)
    out = {"id": a["id"].copy(), "r": a["r"].copy(), "v": a["v"].copy()}
    out["comp"] = (a["cid"].astype(np.int64) - 1) if "cid" in a.dtype.names else np.zeros(n, np.int64)
    out["q"] = a["q"].copy() if "q" in a.dtype.names else np.tile([1.0, 0.0, 0.0, 0.0], (n, 1))
    out["L"] = a["L"].copy() if "L" in a.dtype.names else np.zeros((n, 3))
    return time, box, out


# ---------------------------------------------------------------- Andersen
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z):
    """SplitMix64 output function (Steele, Lea and Flood, OOPSLA 2014) on
    uint64 arrays; arithmetic wraps modulo 2^64."""
    z = np.asarray(z, np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def andersen_control(ids, comp, r, v, L, masses, region, T, nu_dt, seed, step, index):
    """One Andersen collision pass of a TemperatureControl region
    (thermostats/TemperatureControl.cpp:367-379 region and component test,
    :411-419 the collision), with the counter-based draws the engine uses in
    place of the reference's sequential generator: draw k of molecule `id`
    in region `index` at `step` is SplitMix64(key + k) with key =
    mix(mix(mix(seed ^ mix(step)) ^ id) ^ index); draw 0 < nu_dt selects;
    draws 1 + 2d, 2 + 2d are a Box-Muller pair, v_d = g sd, L_d = g' sd,
    sd = sqrt(T / m) (the reference's shared reserve deviate gives L the
    translational deviation).  ``region``: lower, upper (open box) and the
    1-based component (0 = all).  Returns new (v, L) and the selection mask."""
    with np.errstate(over="ignore"):
        ids = np.asarray(ids, np.uint64)
        inside = np.ones(len(ids), bool)
        if region["component"]:
            inside &= np.asarray(comp) + 1 == region["component"]
        for d in range(3):
            inside &= (r[:, d] > region["lower"][d]) & (r[:, d] < region["upper"][d])
        key = _mix64(np.uint64(seed) ^ _mix64(np.uint64(step)))
        key = _mix64(_mix64(key ^ ids) ^ np.uint64(index))

        def uniform(k):
            return (_mix64(key + np.uint64(k)) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53

        sel = inside & (uniform(0) < nu_dt)
        sd = np.sqrt(T / np.asarray(masses, float)[np.asarray(comp)])
        v, L = v.copy(), L.copy()
        for d in range(3):
            rad = np.sqrt(-2.0 * np.log(1.0 - uniform(1 + 2 * d)))
            ang = 2.0 * np.pi * uniform(2 + 2 * d)
            v[sel, d] = (rad * np.cos(ang) * sd)[sel]
            L[sel, d] = (rad * np.sin(ang) * sd)[sel]
    return v, L, sel
