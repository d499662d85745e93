"""Benchmark: molecule-updates/s of the short-range MD step on one GB300.

Workload (default, the precision-form 1CLJ case at scale): single-centre LJ
(eps = sigma = m = 1), fcc 100^3 x 4 = 4,000,000 molecules at rho* = 0.75,
Maxwell-Boltzmann velocities at T* = 0.9 (seeded, net momentum removed),
rc = 3.0 sigma, dt = 0.002, periodic box, NVE Leapfrog, mixed precision (FP32
pair arithmetic, compensated per-molecule sums, FP64 state).  A "step" is one
full MD step: pre-force half step, rebin/halo + pair-candidate list when due,
forces, post-force half step and the Upot/virial/kinetic sums.

  value   molecule-updates/s with the state resident in HBM, device-timed with
          CUDA events on the engine's stream (max over ranks);
  e2e     the same metric through the C ABI from host buffers: upload of the
          phase space, the K steps with the per-step sums read back, and the
          download of the final phase space, all inside the timed region;
  roofline  the pair kernel (dominant kernel) against the FP32 FMA rate:
          the reference's FlopCounter flops of the unique in-cutoff pairs per
          launch / event-timed launch duration, against SMs x 128 lanes x 2
          flop x the SM clock sampled during the timed region (nominal rate
          at that clock; the measured-peaks file holds no FP32 figure);
  roofline_hbm  the same launch as algorithmic bytes against the measured
          HBM copy bandwidth, with the DRAM traffic scaled from an ncu capture;
  precision  mixed vs FP64 at the final state of the timed steps: relative rms
          force error, Upot / virial / pressure errors, pair counts;
  fp64   the same workload through the FP64 kernel (molecule-updates/s), and
          the adjoint / forward pair-kernel time ratio;
  mixture, batch  the 1M 2CLJQ/1CLJD mixture (device-timed steps, the
          multi-site pair kernel's FP32 roofline fraction, its errors against
          FP64) and the 512-box batch (autotuned, device-timed), in short;
  cpu_baseline  the CPU oracle (C restatement of the reference's path, OpenMP
          C08 traversal) on all host cores on the full workload for as many
          steps as fit in a bounded time.

--impl reference times that CPU path alone (rank 0; other ranks exit 0).
Multi-GPU: independent replicas (one box per rank, no collective on the data
path), value = all ranks' updates / max time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ls1-mardyn_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

from ls1gb300 import phasespace as psm  # noqa: E402

WORKLOADS = {
    # name: (generator, rc, dt, description)
    "lj4m": (lambda: psm.lj_fcc(100, 0.75, 0.9, seed=2024), 3.0, 0.002,
             "1CLJ fcc 100^3x4 = 4,000,000, rho*=0.75, T*=0.9, rc=3.0, dt=0.002"),
    "lj1m": (lambda: psm.lj_fcc(63, 0.75, 0.9, seed=2024), 3.0, 0.002,
             "1CLJ fcc 63^3x4 = 1,000,188, rho*=0.75, T*=0.9, rc=3.0, dt=0.002 (profiling size)"),
    "lj32k": (lambda: psm.lj_fcc(20, 0.8, 1.0, seed=1), 2.5, 0.002,
              "1CLJ fcc 20^3x4 = 32,000, rho*=0.8, T*=1.0, rc=2.5, dt=0.002"),
    "slab": (lambda: psm.lj_slab(91, 0.73, 0.02, 0.9, seed=2025), 3.0, 0.002,
             "1CLJ vapour-liquid slab, 3.2M molecules, rho_l*=0.73, rho_v*=0.02, T*=0.9, rc=3.0"),
    "mix1m": (lambda: psm.mixture(1_000_000, 18.0, 300.0, seed=2026), 1.0, 9.118e-5,
              "2CLJQ/1CLJD 50/50 mixture, N=1,000,188, n=18 nm^-3, T=300 K, rc=1 nm, RF eps=1e10, dt=1 fs"),
}
BATCH_DESC = ("512 independent periodic 1CLJ boxes, N log-uniform in [500, 20000] (seeded), rho* U[0.05, 0.85], "
              "T* U[0.7, 1.3], rc=2.5, dt=0.002, graphs of 100 steps, skin and threads per molecule row autotuned")
DEFAULT_SKIN = {"lj4m": 0.25, "lj1m": 0.25, "lj32k": 0.3, "slab": 0.25, "mix1m": 0.1}
FLOP_PER_PAIR_LJ = 39.0  # reference FlopCounter model: 31 per LJ site pair + 8 per molecule distance
# FlopCounter flops per unique interacting site pair, by kind (LJ, C-C, C-D, D-D with RF, C-Q, D-Q, Q-Q), and per
# unique interacting molecule pair for the centre distance (src/utils/FlopCounter.cpp:19-73)
FLOP_PER_SITE_PAIR = (31.0, 24.0, 52.0, 127.0, 69.0, 141.0, 151.0)
FLOP_PER_MOL_PAIR = 8.0
FP32_LANES_PER_SM = 128  # FP32 FMA lanes per SM (4 sub-partitions x 32)
# DRAM bytes (read + write) of one k_force_lj32x2 launch per pair-candidate list entry, from an ncu
# capture of the 1,000,188-molecule case (434.2 MB for 100.2 entries per molecule); traffic grows
# with the entries read, so it is scaled by the live entry count.
FORCE_DRAM_BYTES_PER_ENTRY = 434.15e6 / (1_000_188 * 100.2)
# The same for the pair kernel with both Leapfrog half steps fused (md_run's steps of one component of
# single-centre LJ molecules in mixed precision): 518.4 MB for 105.5 entries per molecule at 1,000,188.
STEP_DRAM_BYTES_PER_ENTRY = 518.4e6 / (1_000_188 * 105.47)
# algorithmic bytes per molecule of that kernel beyond the list entries: position 16, count 4, r and v read
# and written 4 x 24, home-cell origin 24, local coordinates at the list build 16, next local coordinates 16
STEP_BYTES_PER_MOLECULE = 16 + 4 + 4 * 24 + 24 + 16 + 16


# ---------------------------------------------------------------- CUDA events on the engine stream
class Cudart:
    def __init__(self):
        import glob
        cands = sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")) + ["libcudart.so"]
        self.L = None
        for c in cands:
            try:
                self.L = C.CDLL(c)
                break
            except OSError:
                continue
        if self.L is None:
            raise RuntimeError("libcudart not found")
        self.L.cudaEventCreate.argtypes = [C.POINTER(C.c_void_p)]
        self.L.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
        self.L.cudaEventSynchronize.argtypes = [C.c_void_p]
        self.L.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
        self.L.cudaEventDestroy.argtypes = [C.c_void_p]
        self.L.cudaDeviceGetAttribute.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_int]

    def attr(self, which: int, device: int) -> int:
        v = C.c_int()
        assert self.L.cudaDeviceGetAttribute(C.byref(v), which, device) == 0
        return int(v.value)

    def event(self):
        e = C.c_void_p()
        assert self.L.cudaEventCreate(C.byref(e)) == 0
        return e

    def record(self, e, stream):
        assert self.L.cudaEventRecord(e, C.c_void_p(stream)) == 0

    def elapsed_ms(self, a, b) -> float:
        assert self.L.cudaEventSynchronize(b) == 0
        ms = C.c_float()
        assert self.L.cudaEventElapsedTime(C.byref(ms), a, b) == 0
        return float(ms.value)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []      # (time, line) of every sample
        self.t_end = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, wait_s: float = 1.0) -> dict:
        """Samples taken since start(); when the timed region was shorter than
        nvidia-smi's start-up and sampling period, waits (up to wait_s) for the
        first sample, which then describes the clocks right after the region
        (clock locks and throttle reasons persist); `after_region` counts such
        samples."""
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.t_end = time.perf_counter()
        deadline = self.t_end + wait_s
        while not self.lines and time.perf_counter() < deadline:
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        after = sum(1 for t, _ in self.lines if t > self.t_end)
        for _, line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "after_region": after}


# ---------------------------------------------------------------- CPU baseline (oracle)
def cpu_baseline(workload: str, budget_s: float = 20.0, max_steps: int = 10 ** 9, warmup: int = 0) -> dict:
    """The oracle (the C restatement of the reference's path: OpenMP C08
    traversal, scalar loop bodies, Leapfrog) on the full workload with all
    host cores: a first force pass and `warmup` untimed steps, then NVE steps
    one at a time until `budget_s` or `max_steps` is reached (at least 2)."""
    from oracle.oracle import Oracle
    gen, rc, dt, desc = WORKLOADS[workload]
    ps = gen()
    threads = os.cpu_count() or 1
    o = Oracle(ps, rc, threads=threads)
    o.rebin()
    o.forces()
    if warmup:
        o.run(dt, warmup)
    steps, t0 = 0, time.perf_counter()
    while True:
        o.run(dt, 1)
        steps += 1
        el = time.perf_counter() - t0
        if steps >= max_steps or (el > budget_s and steps >= 2):
            break
    return {"value": ps.n * steps / el, "unit": "molecule-updates/s", "cores": threads, "kind": "port",
            "molecules": int(ps.n),
            "sample": f"the full workload ({ps.n:,} molecules); {steps} NVE steps in {el:.1f} s with {threads} "
                      f"OpenMP threads (oracle: C08 cell pairs, scalar loop bodies, FP64)"}


# ---------------------------------------------------------------- main
def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lj4m", choices=sorted(WORKLOADS) + ["batch512", "adjoint"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--skin", type=float, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--pair-scheme", default="auto", choices=["auto", "rows", "newton3"],
                    help="rows: per-molecule candidate rows, each pair from both sides; newton3: every pair once "
                         "where the system allows (cluster pairs for 1CLJ, half rows with atomics for multi-site "
                         "molecules); auto: newton3 for multi-site molecules (measured 1.4x faster), rows for "
                         "single-centre LJ (the cluster pairs measured no faster)")
    ap.add_argument("--integrator", default="leapfrog", choices=["leapfrog", "rmm"],
                    help="rmm: the reduced memory mode (LeapfrogRMM + VCP1CLJRMM, 1CLJ only)")
    return ap.parse_args()


def dist_setup():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_BACKEND", "nccl") == "nccl" else "gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    dev = "cuda" if os.environ.get("BENCH_BACKEND", "nccl") == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(pg, world: int, n_per_rank: int, steps: int, ms_local: float):
    """Whole-job molecule-updates/s of `world` independent replicas (one box
    per rank, no collective on the data path): the updates of all ranks over
    the slowest rank's timed region.  Returns (value, slowest ms)."""
    ms = max_over_ranks(pg, ms_local)
    return world * n_per_rank * steps / (ms * 1e-3), ms


def workload_config(a, desc: str, n: int, skin: float) -> dict:
    """The `config` of the bench line, shared by both arms."""
    return {"workload": desc, "precision": a.precision, "skin": skin, "molecules": n,
            "integrator": "LeapfrogRMM (reduced memory mode)" if a.integrator == "rmm" else "Leapfrog",
            "parallelism": "replicas x1" if a.gpus == 1 else f"replicas x{a.gpus}",
            "l2": "working set > L2 (GBs), no flush needed"}


def run_reference(a, rank):
    """The reference's CPU path for this workload (the oracle port; the
    reference tree itself is not on the GPU host) on the full workload, all
    host cores: min(W, 1) untimed steps, then up to K timed steps within a
    bounded time."""
    if rank != 0:
        return
    gen, rc, dt, desc = WORKLOADS[a.workload]
    skin = DEFAULT_SKIN[a.workload] if a.skin is None else a.skin
    cb = cpu_baseline(a.workload, budget_s=120.0, max_steps=a.steps, warmup=min(a.warmup, 1))
    n = cb["molecules"]
    line = {"impl": "reference", "metric": "molecule-updates/s", "value": cb["value"], "unit": "molecule-updates/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded fcc lattice, Maxwell-Boltzmann velocities)",
            "config": workload_config(a, desc, n, skin),
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "molecule-updates/s",
                                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def batch_cpu_baseline(boxes, budget_s: float = 12.0) -> dict:
    from oracle.oracle import Oracle
    threads = os.cpu_count() or 1
    done, t0, used = 0, time.perf_counter(), []
    for b in boxes:
        o = Oracle(b.to_phasespace(rc=2.5), 2.5, threads=threads)
        o.rebin()
        o.forces()
        o.run(0.002, 20)
        done += 20 * b.n
        used.append(b.n)
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": done / el, "unit": "molecule-updates/s", "cores": threads, "kind": "port",
            "sample": f"the first {len(used)} boxes of the batch ({sum(used)} molecules), 20 NVE steps each, one at a "
                      f"time, {el:.1f} s with {threads} OpenMP threads"}


def run_batch(a, rank, world, local, pg):
    """Batch of independent boxes: md_batch throughput, per-box errors of the
    mixed batch against the FP64 batch, and the same boxes run one at a time
    through md_ctx in FP64 on the same GPU (a sample of them, timed)."""
    from ls1gb300 import batch as B
    from ls1gb300 import engine as E
    cu = Cudart()
    boxes = B.random_boxes(512, 500, 20000, seed=2024 + rank)
    n = sum(b.n for b in boxes)
    dt = 0.002
    bt = B.Batch(boxes, 2.5, precision="mixed", device=local)
    bt.forces()
    tune = bt.autotune(dt, trial_steps=30)
    bt.forces()
    bt.run(dt, max(3, a.warmup), graph_steps=100, record=False)
    stream = bt.stream()
    clock = ClockSampler(local)
    barrier(pg)
    e0, e1 = cu.event(), cu.event()
    rb0 = bt.rebuilds()
    clock.start()
    cu.record(e0, stream)
    rec = bt.run(dt, a.steps, graph_steps=100, record=True)
    cu.record(e1, stream)
    ms = cu.elapsed_ms(e0, e1)
    clocks = clock.stop()
    rebuilds = bt.rebuilds()
    rebuilds_timed = rebuilds - rb0
    value, ms = replica_throughput(pg, world, n, a.steps, ms)
    # per-box errors of the mixed batch at its final state: Upot and pressure
    # p = (sum m v^2 + virial) / (3 V) from the last step's record against the
    # FP64 forces of the same positions
    fin = bt.molecules()
    bt.close()
    fboxes = [B.Box(L=b.L, r=np.ascontiguousarray(fin["r"][o:e]), v=np.ascontiguousarray(fin["v"][o:e]), rho=b.rho,
                    T=b.T) for b, o, e in zip(boxes, bt.box_start[:-1], bt.box_start[1:])]
    ref = B.Batch(fboxes, 2.5, precision="fp64", skin=0.3, device=local)
    s64 = ref.forces()
    ref.close()
    vol = np.array([np.prod(b.L) for b in boxes])
    nb = np.array([b.n for b in boxes], dtype=np.float64)
    last = rec[-1]
    du = np.abs(last[:, 0] - s64[:, 0]) / np.maximum(np.abs(s64[:, 0]), 1e-300)
    p64 = (last[:, 2] + s64[:, 1]) / (3.0 * vol)
    dp = np.abs(last[:, 1] - s64[:, 1]) / (3.0 * vol) / np.abs(p64)
    # end to end through the C ABI: create + upload + first forces + K steps (per-step per-box sums) + download
    t0 = time.perf_counter()
    bt2 = B.Batch(boxes, 2.5, precision="mixed", skin=tune["skin"], threads_per_molecule=tune["threads_per_molecule"],
                  cell_occupancy=tune["cell_occupancy"],
                  device=local)
    bt2.forces()
    rec2 = bt2.run(dt, a.steps, graph_steps=100, record=True)
    out = bt2.molecules()
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
    bt2.close()
    h2d = n * 6 * 8 + n * 8 + 8 * (len(boxes) + 1)
    d2h = rec2.nbytes + sum(out[k].nbytes for k in out)
    # one box at a time, FP64 md_ctx on the same GPU: a spread sample of 16 boxes, 100 steps each
    order = np.argsort(nb)
    sample = [int(order[k]) for k in np.linspace(0, len(boxes) - 1, 16).astype(int)]
    upd, tot_ms = 0, 0.0
    for k in sample:
        eng = E.Engine(boxes[k].to_phasespace(rc=2.5), 2.5, precision="fp64", skin=0.3, device=local)
        eng.forces()
        eng.run(dt, 10, record=False)
        st = eng.stream()
        c0, c1 = cu.event(), cu.event()
        cu.record(c0, st)
        eng.run(dt, 100, record=True)
        cu.record(c1, st)
        tot_ms += cu.elapsed_ms(c0, c1)
        upd += boxes[k].n * 100
        eng.close()
    seq = upd / (tot_ms * 1e-3)
    # what one persistent launch per chunk could save: the graph's per-node launch cost (4 nodes per step: the
    # rebuild test, the conditional rebuild node, the pair kernel with both half steps, the box sums), and
    # the time the largest box would need on one SM at the measured per-SM rate (one box per block)
    node_us = graph_node_us(local)
    step_us = 1e3 * ms / a.steps
    nmax = max(b.n for b in boxes)
    persistent = {"graph_node_us": node_us, "nodes_per_step": 4, "step_us": step_us,
                  "launch_share_of_step": 4 * node_us / step_us, "largest_box": nmax,
                  "largest_box_on_one_sm_us": step_us * cu.attr(16, local) * nmax / n}  # 16: SM count
    cb = batch_cpu_baseline(boxes) if (rank == 0 and world == 1 and not a.no_cpu_baseline) else None
    if rank == 0:
        line = {
            "metric": "molecule-updates/s", "value": value, "unit": "molecule-updates/s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-pairs/f64-state",
            "data": "synthetic (seeded boxes on fcc sites, Maxwell-Boltzmann velocities)",
            "config": {"workload": BATCH_DESC, "boxes": len(boxes), "molecules": n, "precision": "mixed",
                       "autotune": tune, "parallelism": f"replicas x{world}",
                       "l2": "working set > L2 (state + lists of 2.7M molecules), no flush needed"},
            # per step: pre, check, force, post, box sums; 11 more in a step that rebuilds the list (a conditional
            # node of the step graph)
            "gpu_launches": 5 * a.steps + 11 * rebuilds_timed,
            "batch": {"rebuilds": rebuilds,
                      "errors_vs_fp64": "per box at the final state: Upot from the last step's record and the "
                                        "pressure (sum m v^2 + virial) / 3V against FP64 forces of the same positions",
                      "upot_rel_err_max": float(du.max()), "upot_rel_err_median": float(np.median(du)),
                      "pressure_rel_err_max": float(dp.max()), "pressure_rel_err_median": float(np.median(dp)),
                      "one_at_a_time_fp64": {"value": seq, "unit": "molecule-updates/s",
                                             "sample": "16 boxes spread over the N range, md_ctx FP64, 100 steps each"},
                      "speedup_vs_one_at_a_time_fp64": value / seq,
                      "persistent_launch_bound": persistent},
            "clocks": clocks,
            "e2e": {"value": world * n * a.steps / e2e_s, "unit": "molecule-updates/s",
                    "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps},
            "cpu_baseline": cb,
        }
        print(json.dumps(line))


def graph_node_us(device: int, nodes: int = 400) -> float:
    """Per-node cost of a replayed CUDA graph of `nodes` dependent one-block
    kernels (torch capture; best of 20 replays), the launch cost that one
    persistent kernel per chunk would save."""
    import torch
    x = torch.zeros(256, device=f"cuda:{device}")
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream(device=device)
    with torch.cuda.stream(s):
        x.add_(1.0)
        torch.cuda.synchronize(device)
        with torch.cuda.graph(g, stream=s):
            for _ in range(nodes):
                x.add_(1.0)
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(20):
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize(device)
        best = min(best, e0.elapsed_time(e1))
    return best * 1e3 / nodes


def is_multisite(ps) -> bool:
    """Whether any component is more than one LJ centre at its origin."""
    return any(len(c.lj) != 1 or c.charges or c.dipoles or c.quadrupoles or any(x != 0 for x in c.lj[0].r)
               for c in ps.components)


def scheme_for(choice: str, ps) -> str:
    """The pair scheme a run uses: the choice, or for "auto" Newton-3 for
    multi-site molecules and the rows for single-centre LJ."""
    if choice != "auto":
        return choice
    return "newton3" if is_multisite(ps) else "rows"


def mixture_summary(local: int, steps: int = 20) -> dict:
    """The 1M 2CLJQ/1CLJD mixture (the mix1m workload) in short: device-timed
    NVE steps after a warm-up in the multi-site kernels' Newton-3 form (every
    molecule pair once) and with the rows (every pair from both sides), the
    pair kernel's time and FP32 roofline fraction, and the Newton-3 form's
    mixed-precision errors against FP64."""
    from ls1gb300 import engine as E
    from ls1gb300 import precision as P
    cu = Cudart()
    gen, rc, dt, desc = WORKLOADS["mix1m"]
    ps = gen()
    skin = DEFAULT_SKIN["mix1m"]
    sms, mhz = cu.attr(16, local), cu.attr(13, local) / 1e3
    peak = sms * FP32_LANES_PER_SM * 2 * mhz * 1e6 / 1e12
    res = {}
    for scheme in ("newton3", "rows"):
        e = E.Engine(ps, rc, precision="mixed", skin=skin, device=local, pair_scheme=scheme)
        e.forces()
        e.run(dt, 5, record=False)
        st = e.stream()
        c0, c1 = cu.event(), cu.event()
        cu.record(c0, st)
        e.run(dt, steps, record=True)
        cu.record(c1, st)
        ms = cu.elapsed_ms(c0, c1)
        fo = e.forces()
        kt = e.time_kernels(5)
        mol = e.molecules()
        e.close()
        flops = FLOP_PER_MOL_PAIR * fo.mol_pairs + sum(f * k for f, k in zip(FLOP_PER_SITE_PAIR, fo.site_pairs))
        tflops = flops / (kt.force_ms * 1e-3) / 1e12
        res[scheme] = {"pair_scheme": scheme, "value": ps.n * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                       "pair_kernel_ms": kt.force_ms, "pair_kernel_tflops": tflops,
                       "pair_kernel_frac_fp32": tflops / peak}
        if scheme == "newton3":
            assert kt.pair_scheme == 1
            res[scheme]["precision"] = P.report(P.state_of(mol, ps), rc, skin=skin, device=local,
                                                mixed_forces=(fo, mol))
    out = {"workload": desc, "molecules": ps.n, "unit": "molecule-updates/s", "steps": steps,
           "fp32_peak_note": "nominal FP32 FMA rate at the device's maximum clock"}
    out.update(res["newton3"])
    out["rows"] = res["rows"]
    return out


def batch_summary(local: int, steps: int = 100) -> dict:
    """The 512-box batch (the batch512 workload) in short: autotuned, then
    device-timed steps in graphs of 100."""
    from ls1gb300 import batch as B
    cu = Cudart()
    boxes = B.random_boxes(512, 500, 20000, seed=2024)
    n = sum(b.n for b in boxes)
    dt = 0.002
    bt = B.Batch(boxes, 2.5, precision="mixed", device=local)
    bt.forces()
    tune = bt.autotune(dt, trial_steps=30)
    bt.forces()
    bt.run(dt, 10, graph_steps=100, record=False)
    st = bt.stream()
    c0, c1 = cu.event(), cu.event()
    cu.record(c0, st)
    bt.run(dt, steps, graph_steps=100, record=True)
    cu.record(c1, st)
    ms = cu.elapsed_ms(c0, c1)
    bt.close()
    return {"workload": BATCH_DESC, "boxes": len(boxes), "molecules": n, "value": n * steps / (ms * 1e-3),
            "unit": "molecule-updates/s", "ms_per_step": ms / steps, "steps": steps, "autotune": tune}


def _perturbed(ps, f: float):
    """The phase space with every LJ eps, sigma and multipole magnitude scaled by f."""
    import copy
    q = ps.copy()
    comps = copy.deepcopy(ps.components)
    for c in comps:
        for s in c.lj:
            s.eps *= f
            s.sigma *= f
        for s in c.dipoles + c.quadrupoles:
            s.abs *= f
    q.components = comps
    return q


def run_adjoint(a, rank, world, local, pg):
    """Forward and adjoint cost on the differentiation workload: 64 snapshots
    each of 1CLJ (100,000 molecules: fcc 30^3 x 4 with 8,000 seeded vacancies,
    rho*=0.7, T*=1.1, rc=2.5) and of the 2CLJQ/1CLJD mixture (100,000 molecules
    the same way, 18 nm^-3, rc=1 nm).  Per snapshot the loss is
    L = (U - U*)^2 + w (P - P*)^2 with targets from the FP64 forward at +2 %
    parameters; the forward is md_compute_forces (list build + pair kernel +
    sums), the adjoint md_adjoint (pairs recomputed from the list; gradients
    of L w.r.t. positions and eps, sigma, |Q|, |mu|), FP32 pair arithmetic with
    FP64 accumulation."""
    from ls1gb300 import engine as E
    cu = Cudart()
    systems = [("1CLJ N=100,000 (fcc 30^3x4 with 8,000 vacancies), rho*=0.7, T*=1.1, rc=2.5",
                psm.with_vacancies(psm.lj_fcc(30, 0.7, 1.1, seed=4), 100_000, 0.7, 4), 2.5, 0.002, 0.3),
               ("2CLJQ/1CLJD mixture N=100,000 (fcc 30^3x4 with 8,000 vacancies), n=18 nm^-3, T=300 K, rc=1 nm",
                psm.with_vacancies(psm.mixture(108_000, 18.0, 300.0, seed=4), 100_000, 18.0, 4), 1.0, 9.118e-5,
                0.1)]
    out = []
    for desc, ps, rc, dt, skin in systems:
        n = ps.n
        vol = float(np.prod(ps.box))
        eng = E.Engine(ps, rc, precision="mixed", skin=skin, device=local)
        eng.forces()
        snaps = []
        for _ in range(64):
            eng.run(dt, 20, record=False)
            snaps.append(eng.molecules())
        eng.close()
        w = 1.0
        fwd, adj, losses = [], [], []
        tgt_ps = _perturbed(ps, 1.02)
        scheme = scheme_for(a.pair_scheme, ps)
        ev = E.Engine(ps, rc, precision="mixed", skin=skin, device=local, pair_scheme=scheme)
        et = E.Engine(tgt_ps, rc, precision="fp64", skin=skin, device=local)
        st = ev.stream()
        for m in snaps:
            for e_, ps_ in ((ev, ps), (et, tgt_ps)):
                q = ps_.copy()
                order = np.argsort(m["ids"])
                q.r, q.v, q.q, q.L = m["r"][order], m["v"][order], m["q"][order], m["L"][order]
                q.ids, q.comp = m["ids"][order], m["comp"][order]
                e_.upload(q)
            ft = et.forces()
            u_t, p_t = ft.upot, ft.virial / (3 * vol)
            c0, c1, c2 = cu.event(), cu.event(), cu.event()
            cu.record(c0, st)
            fo = ev.forces()
            cu.record(c1, st)
            gu = 2.0 * (fo.upot - u_t)
            gw = 2.0 * w * (fo.virial / (3 * vol) - p_t) / (3 * vol)
            ev.adjoint(gu, gw)
            cu.record(c2, st)
            fwd.append(cu.elapsed_ms(c0, c1))
            adj.append(cu.elapsed_ms(c1, c2))
            losses.append((fo.upot - u_t) ** 2 + w * (fo.virial / (3 * vol) - p_t) ** 2)
        kt = ev.time_kernels(10)
        ev.close()
        et.close()
        f_ms, a_ms = float(np.mean(fwd[4:])), float(np.mean(adj[4:]))
        out.append({"system": desc, "molecules": n, "snapshots": len(snaps), "pair_scheme": scheme,
                    "call_forward_ms": f_ms, "call_adjoint_ms": a_ms, "call_adjoint_over_forward": a_ms / f_ms,
                    "kernel_forward_ms": kt.force_ms, "kernel_adjoint_ms": kt.adjoint_ms,
                    "adjoint_over_forward": kt.adjoint_ms / kt.force_ms, "mean_loss": float(np.mean(losses))})
    if rank == 0:
        print(json.dumps({"metric": "adjoint/forward cost", "value": max(o["adjoint_over_forward"] for o in out),
                          "unit": "ratio", "higher_is_better": False, "n_gpus": world,
                          "dtype": "f32-pairs/f64-accumulation", "data": "synthetic (seeded snapshots of NVE runs)",
                          "config": {"workload": "64 snapshots each of 1CLJ N=100,000 and the 2CLJQ/1CLJD mixture "
                                                 "N=100,000; loss (U-U*)^2 + w (P-P*)^2, targets from FP64 at +2 % "
                                                 "parameters; CUDA events on the engine stream",
                                     "value": "max over the two systems of adjoint pair-kernel time / forward "
                                              "pair-kernel time on the same list; call_* are the whole ABI calls "
                                              "per snapshot (md_compute_forces with its list build vs md_adjoint "
                                              "with the n x 3 gradient copied to the host)"},
                          "systems": out}))


def main():
    a = parse()
    rank, world, local, pg = dist_setup()
    if a.impl == "reference":
        run_reference(a, rank)
        return
    if a.workload in ("batch512", "adjoint"):
        import build as engine_build
        if rank == 0:
            engine_build.build()
        barrier(pg)
        (run_batch if a.workload == "batch512" else run_adjoint)(a, rank, world, local, pg)
        if pg is not None:
            pg.destroy_process_group()
        return
    import build as engine_build
    if rank == 0:
        engine_build.build()
    barrier(pg)
    from ls1gb300 import engine as E

    gen, rc, dt, desc = WORKLOADS[a.workload]
    skin = DEFAULT_SKIN[a.workload] if a.skin is None else a.skin
    ps = gen()
    n = ps.n
    cu = Cudart()

    # ---- device-resident timing
    rmm = a.integrator == "rmm"
    # md_run fuses Leapfrog's half steps into the pair kernel for one component of single-centre LJ molecules in
    # mixed precision
    fused = (a.precision == "mixed" and len(ps.components) == 1 and len(ps.components[0].lj) == 1
             and not (ps.components[0].charges or ps.components[0].dipoles or ps.components[0].quadrupoles))
    mass = ps.components[0].lj[0].m if rmm else 1.0

    def first_forces(e):
        return e.rmm_forces(0.5 * dt / mass) if rmm else e.forces()

    def steps(e, k, record):
        return e.rmm_run(dt, k, record=record) if rmm else e.run(dt, k, record=record)

    scheme = scheme_for(a.pair_scheme, ps)
    eng = E.Engine(ps, rc, precision=a.precision, skin=skin, device=local, pair_scheme=scheme)
    fo0 = first_forces(eng)
    steps(eng, max(3, a.warmup), False)
    eng.sync()
    stream = eng.stream()
    t_clock = ClockSampler(local)
    barrier(pg)
    e0, e1 = cu.event(), cu.event()
    rb0 = eng.rebuilds()
    t_clock.start()
    cu.record(e0, stream)
    steps(eng, a.steps, True)
    cu.record(e1, stream)
    ms = cu.elapsed_ms(e0, e1)
    clocks = t_clock.stop()
    rebuilds_timed = eng.rebuilds() - rb0
    value, ms = replica_throughput(pg, world, n, a.steps, ms)
    # per-kernel times on the engine stream, right after the timed region
    fo = eng.forces()
    mol = eng.molecules()
    kt = eng.time_kernels(5)
    # precision at the final state of the timed steps: the same positions through the FP64 kernel
    from ls1gb300 import precision as P
    prec = None
    if a.precision == "mixed" and not rmm:
        prec = P.report(P.state_of(mol, ps), rc, skin=skin, device=local, mixed_forces=(fo, mol))
    multisite = not (len(ps.components) == 1 and len(ps.components[0].lj) == 1
                     and not (ps.components[0].charges or ps.components[0].dipoles or ps.components[0].quadrupoles))
    pairs = fo.site_pairs[0]
    if multisite:
        flops = FLOP_PER_MOL_PAIR * fo.mol_pairs + sum(f * k for f, k in zip(FLOP_PER_SITE_PAIR, fo.site_pairs))
        flop_desc = (f"FlopCounter model: 8 flop x {fo.mol_pairs} unique interacting molecule pairs + per site-pair "
                     f"kind (LJ 31, C-C 24, C-D 52, D-D 127, C-Q 69, D-Q 141, Q-Q 151) x {list(fo.site_pairs)}")
    else:
        flops = FLOP_PER_PAIR_LJ * pairs
        flop_desc = f"FlopCounter model: {FLOP_PER_PAIR_LJ:.0f} flop x {pairs} unique in-cutoff LJ pairs per launch"
    list_bytes = kt.mean_candidates * n * 4.0
    # the dominant kernel of the timed steps: in the fused Leapfrog steps the pair kernel that also runs
    # both half steps, else the plain pair kernel
    n3 = kt.pair_scheme == 1
    step_kernel = fused and not rmm and kt.step_force_ms > 0 and not n3
    ms_name = ("k_force_ms2<float, SigMixA, SigMixB" if a.workload == "mix1m" else "k_force_ms<float") \
        if a.precision == "mixed" else ("k_force_ms2<double, SigMixA, SigMixB" if a.workload == "mix1m"
                                        else "k_force_ms<double")
    if n3 and multisite:
        kname = ms_name + ", N3> (Newton-3: higher-slot half rows, the neighbour's share by vector atomics)"
        launch_ms = kt.force_ms
        hbm_bytes = 0.5 * list_bytes + n * (16 + 4 + 4 + 9 * 8 + 3 * 16)
        alg_desc = ("per launch: 4 B per entry of the half rows + 16 B position + 8 B counts + 72 B F/M/Vi + "
                    "48 B accumulators per molecule")
        traffic = None
    elif n3:
        kname = f"k_force_n3 (Newton-3 cluster pairs, {kt.cluster_size} molecules per cluster)"
        launch_ms = kt.force_ms
        ncl = n / kt.cluster_size
        hbm_bytes = list_bytes + n * (16 + 32) + ncl * 12
        alg_desc = ("per launch: 4 B per cluster-list entry + 16 B position + 32 B force accumulator (read and "
                    "written) per molecule + 12 B cluster record and list length per cluster")
        traffic = None
    elif step_kernel:
        kname = "k_force_lj32x2<EPI_LEAPFROG> (pair kernel with both Leapfrog half steps)"
        launch_ms = kt.step_force_ms
        hbm_bytes = list_bytes + n * STEP_BYTES_PER_MOLECULE
        alg_desc = ("per launch: 4 B per pair-candidate list entry + 16 B position + 4 B count + 152 B Leapfrog "
                    "state per molecule (r and v read and written, home-cell origin, list-build and next local "
                    "coordinates)")
        traffic = STEP_DRAM_BYTES_PER_ENTRY * kt.mean_candidates * n
    else:
        if multisite:
            kname = ms_name + ">"
        else:
            kname = "k_force_lj32x2" if a.precision == "mixed" else "k_force_lj64"
        launch_ms = kt.force_ms
        hbm_bytes = list_bytes + n * (16 + 4 + 9 * 8)
        alg_desc = "per launch: 4 B per pair-candidate list entry + 16 B position + 4 B count + 72 B F/M/Vi per molecule"
        traffic = (FORCE_DRAM_BYTES_PER_ENTRY * kt.mean_candidates * n
                   if a.precision == "mixed" and not multisite else None)
    achieved = flops / (launch_ms * 1e-3) / 1e12
    sms = cu.attr(16, local)                       # cudaDevAttrMultiProcessorCount
    max_mhz = cu.attr(13, local) / 1e3             # cudaDevAttrClockRate (kHz)
    sm_mhz = clocks.get("sm_mhz") or max_mhz
    if clocks.get("sm_max_mhz") is None:  # no nvidia-smi sample: the device's own maximum clock
        clocks["sm_max_mhz"] = max_mhz
        clocks["sm_max_source"] = "device attribute"
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    fp64_lane_note = "FP64 kernel: bound by GB300's FP64 rate, not FP32" if a.precision == "fp64" else None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, hbm_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        hbm_peak, hbm_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    # adjoint / forward pair-kernel time on this context (1CLJ at full size)
    adj = {"system": desc, "kernel_forward_ms": kt.force_ms, "kernel_adjoint_ms": kt.adjoint_ms,
           "adjoint_over_forward": kt.adjoint_ms / kt.force_ms}
    eng.close()

    # ---- the FP64 kernel on the same workload (the engine's own FP64 throughput)
    fp64 = None
    if a.precision == "mixed" and not rmm:
        e64 = E.Engine(ps, rc, precision="fp64", skin=skin, device=local)
        e64.forces()
        e64.run(dt, 3, record=False)
        st64 = e64.stream()
        c0, c1 = cu.event(), cu.event()
        k64 = 10
        cu.record(c0, st64)
        e64.run(dt, k64, record=False)
        cu.record(c1, st64)
        ms64 = cu.elapsed_ms(c0, c1)
        e64.close()
        fp64 = {"value": n * k64 / (ms64 * 1e-3), "unit": "molecule-updates/s", "steps": k64,
                "ms_per_step": ms64 / k64, "mixed_over_fp64": value / (n * k64 / (ms64 * 1e-3))}
    # the Newton-3 cluster-pair path on the same workload (every pair evaluated once), device-timed like `value`
    newton3 = None
    if fused and not rmm and scheme == "rows":
        e3 = E.Engine(ps, rc, precision=a.precision, skin=skin, device=local, pair_scheme="newton3")
        e3.forces()
        e3.run(dt, max(3, a.warmup), record=False)
        st3 = e3.stream()
        c0, c1 = cu.event(), cu.event()
        rb3 = e3.rebuilds()
        cu.record(c0, st3)
        e3.run(dt, a.steps, record=False)
        cu.record(c1, st3)
        ms3 = cu.elapsed_ms(c0, c1)
        rb3 = e3.rebuilds() - rb3
        f3 = e3.forces()
        kt3 = e3.time_kernels(5)
        e3.close()
        a3 = FLOP_PER_PAIR_LJ * f3.site_pairs[0] / (kt3.force_ms * 1e-3) / 1e12
        newton3 = {"value": n * a.steps / (ms3 * 1e-3), "unit": "molecule-updates/s", "ms_per_step": ms3 / a.steps,
                   "kernel": f"k_force_n3 ({kt3.cluster_size} molecules per cluster) + k_n3_lf (both half steps)",
                   "pair_kernel_ms": kt3.force_ms, "half_steps_ms": kt3.lf_ms, "rebuild_ms": kt3.rebuild_ms,
                   "rebuilds_timed": int(rb3), "list_entries_per_molecule": kt3.mean_candidates,
                   "pair_kernel_tflops": a3, "pair_kernel_frac_fp32": a3 / fp32_peak}
    # the adjoint on the differentiation workload's mixture (2CLJQ/1CLJD, 100,000 molecules)
    adj_mix = None
    if a.workload == "lj4m" and a.precision == "mixed" and not rmm:
        mps = psm.with_vacancies(psm.mixture(108_000, 18.0, 300.0, seed=4), 100_000, 18.0, 4)
        ktm = {}
        for mscheme in ("rows", "newton3"):
            em = E.Engine(mps, 1.0, precision="mixed", skin=0.1, device=local, pair_scheme=mscheme)
            em.forces()
            em.run(9.118e-5, 200, record=False)  # off the lattice, as the differentiation workload's snapshots
            ktm[mscheme] = em.time_kernels(5)
            em.close()
        adj_mix = {"system": f"2CLJQ/1CLJD mixture, {mps.n:,} molecules, n=18 nm^-3, T=300 K, rc=1 nm, after 200 steps",
                   "kernel_forward_ms": ktm["rows"].force_ms, "kernel_adjoint_ms": ktm["rows"].adjoint_ms,
                   "adjoint_over_forward": ktm["rows"].adjoint_ms / ktm["rows"].force_ms,
                   "kernel_forward_newton3_ms": ktm["newton3"].force_ms,
                   "adjoint_over_forward_newton3": ktm["newton3"].adjoint_ms / ktm["newton3"].force_ms}

    # the multi-site mixture and the box batch in short, so that one default run records every workload's figure
    mixture, batch = None, None
    if a.workload == "lj4m" and a.precision == "mixed" and not rmm and world == 1:
        mixture = mixture_summary(local)
        batch = batch_summary(local)

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not a.no_e2e:
        # the caller's buffers: page-locked input arrays and output arrays, made before the timed region
        from ls1gb300 import pinned
        host_in = tuple(pinned.copy(x) for x in E.abi.molecule_arrays(ps))
        ids, comp, r, v, q, Lm = host_in
        host_out = {k: pinned.empty(shp, dt) for k, shp, dt in
                    (("ids", (n,), np.uint64), ("comp", (n,), np.int32), ("r", (n, 3), np.float64),
                     ("v", (n, 3), np.float64), ("q", (n, 4), np.float64), ("L", (n, 3), np.float64),
                     ("F", (n, 3), np.float64), ("M", (n, 3), np.float64), ("Vi", (n, 3), np.float64))}
        t0 = time.perf_counter()
        eng2 = E.Engine(ps, rc, precision=a.precision, skin=skin, device=local, pair_scheme=scheme,
                        arrays=host_in)
        t_up = time.perf_counter()
        first_forces(eng2)
        t_f = time.perf_counter()
        rec = steps(eng2, a.steps, True)
        t_run = time.perf_counter()
        out = eng2.molecules(host_out)
        t1 = time.perf_counter()
        e2e_s = max_over_ranks(pg, t1 - t0)
        eng2.close()
        phases = {"create_upload_s": t_up - t0, "first_forces_s": t_f - t_up, "steps_s": t_run - t_f,
                  "download_s": t1 - t_run}
        h2d = sum(x.nbytes for x in (ids, comp, r, v, q, Lm))
        d2h = sum(out[k].nbytes for k in out) + rec.nbytes
        phases["upload_gbs"] = h2d / phases["create_upload_s"] / 1e9
        phases["download_gbs"] = sum(out[k].nbytes for k in out) / phases["download_s"] / 1e9
        e2e = {"value": world * n * a.steps / e2e_s, "unit": "molecule-updates/s",
               "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps,
               "scope": "md_create + upload + first forces + K steps (per-step sums read back) + download, from "
                        "and into the caller's page-locked host arrays",
               "phases": phases}

    cb = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        cb = cpu_baseline(a.workload)
        cb.pop("molecules", None)

    if rank == 0:
        line = {
            "metric": "molecule-updates/s", "value": value, "unit": "molecule-updates/s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-pairs/f64-state" if a.precision == "mixed" else "f64",
            "data": "synthetic (seeded fcc lattice, Maxwell-Boltzmann velocities)",
            "config": workload_config(a, desc, n, skin),
            # graph-captured chunks of 25 steps: the per-step kernels, the rebuild kernels of the steps that
            # rebuilt the list, and per chunk the half steps that are not fused (mixed single-centre LJ: the
            # first pre-force and the last post-force half step; otherwise the first pre-force one); the reduced
            # memory mode runs rebuild test, pair kernel and two finalize launches per step, with the drift in
            # the pair kernel but for the first step of a chunk in mixed precision, as a kernel of its own in FP64
            "gpu_launches": int(((4 if a.precision == "mixed" else 5) if rmm else kt.launches_per_step) * a.steps
                                + kt.launches_per_rebuild * rebuilds_timed
                                + ((1 if a.precision == "mixed" else 0) if rmm else (2 if fused else 1))
                                * -(-a.steps // 25)),
            "roofline": {"bound": "fp32", "kernel": kname, "achieved": achieved, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                         "peak_source": (f"nominal FP32 FMA rate at the sampled SM clock: {sms} SMs (device) x "
                                         f"{FP32_LANES_PER_SM} lanes x 2 flop x {sm_mhz:.0f} MHz"),
                         "algorithmic": flop_desc, "algorithmic_flops": flops, "launch_ms": launch_ms,
                         "note": fp64_lane_note},
            "roofline_hbm": {"bound": "hbm", "kernel": kname,
                             "achieved": hbm_bytes / (launch_ms * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "frac": hbm_bytes / (launch_ms * 1e-3) / 1e9 / hbm_peak,
                             "traffic": traffic, "peak_source": hbm_src,
                             "algorithmic": alg_desc, "algorithmic_bytes": hbm_bytes, "launch_ms": launch_ms},
            "pair_scheme": scheme,
            "precision": prec,
            "fp64": fp64,
            "newton3": newton3,
            "mixture": mixture,
            "batch": batch,
            "adjoint": {"lj": adj, "mixture": adj_mix,
                        # the largest of the reported ratios (1CLJ; the mixture on rows and on its Newton-3 form,
                        # the form its workloads run on by default)
                        "value": max([x["adjoint_over_forward"] for x in (adj, adj_mix) if x]
                                     + ([adj_mix["adjoint_over_forward_newton3"]] if adj_mix else [])),
                        "unit": "adjoint / forward pair-kernel time"},
            "kernels_ms": {"force": kt.force_ms, "force_with_both_half_steps": kt.step_force_ms,
                           "half_steps_after_pairs": kt.lf_ms, "pre": kt.pre_ms, "post": kt.post_ms,
                           "rebuild": kt.rebuild_ms},
            "pair_list": {"scheme": "cluster pairs (every pair once)" if n3 else "per-molecule rows",
                          "entries_per_molecule": kt.mean_candidates, "rebuilds": int(kt.rebuilds),
                          "rebuilds_timed": int(rebuilds_timed)},
            "physics": {"upot_per_molecule": fo.upot / n, "unique_lj_pairs": int(pairs),
                        "unique_molecule_pairs": int(fo.mol_pairs)},
            "clocks": clocks,
            "e2e": e2e,
            "cpu_baseline": cb,
        }
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
