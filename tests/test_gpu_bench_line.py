"""The benchmark line bench.py prints on the GPU (the 32,000-molecule box,
5 timed steps after 3 warm-up steps): every key of the contract is there
and consistent -- whole-job throughput over the timed steps, the roofline
of the dominant kernel (frac = achieved / peak), a CPU baseline of the
oracle on host cores, an end-to-end figure through the C ABI with the host
copies counted, the clocks sampled during the timed steps and the number
of the engine's kernel launches in them."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_line_keeps_the_contract():
    p = subprocess.run([sys.executable, "bench.py", "--workload", "lj32k", "--steps", "5", "--warmup", "3"], cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches"):
        assert k in d, k
    assert d["metric"] == "molecule-updates/s" and d["unit"] == d["metric"] and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 5 and d["warmup"] == 3 and d["scaling"] == "weak"
    n = d["config"]["molecules"]
    assert n == 32000 and "workload" in d["config"]
    assert abs(d["value"] - n * d["steps"] / (d["ms_per_step"] * d["steps"] * 1e-3)) <= 1e-6 * d["value"]
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["peak"] > 0 and r["achieved"] > 0 and abs(r["frac"] - r["achieved"] / r["peak"]) <= 1e-9
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["unit"] == d["unit"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] > 0 and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    c = d["clocks"]
    assert c["sm_max_mhz"] > 0 and isinstance(c["reasons"], list)
    assert d["gpu_launches"] >= d["steps"]
