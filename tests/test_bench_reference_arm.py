"""bench.py's reference arm (`--impl reference`, CPU only): the line it
prints keeps the contract -- impl, the arm's metric and unit, a
cpu_baseline describing the run whose value is the line's, an e2e with no
host<->device bytes, and the same config as the GPU arm -- and under
torch.distributed.run with two ranks only rank 0 prints it while the other
exits 0 without work.  Run on the 32,000-molecule box (one step)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["bench.py", "--impl", "reference", "--workload", "lj32k", "--steps", "1", "--warmup", "1"]


def _json_lines(out: str):
    return [json.loads(x) for x in out.splitlines() if x.startswith("{")]


def _check(line: dict, world: int):
    assert line["impl"] == "reference"
    assert line["metric"] == "molecule-updates/s" and line["unit"] == "molecule-updates/s"
    assert line["higher_is_better"] is True and line["n_gpus"] == world
    assert line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["config"]["molecules"] == 32000


def test_reference_arm_line():
    p = subprocess.run([sys.executable] + ARGS, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = _json_lines(p.stdout)
    assert len(lines) == 1
    _check(lines[0], 1)


def test_reference_arm_two_ranks_print_once():
    pytest.importorskip("torch")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port)] + ARGS[:1] + ["--gpus", "2"] + ARGS[1:]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = _json_lines(p.stdout)
    assert len(lines) == 1
    _check(lines[0], 2)
