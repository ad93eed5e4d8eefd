"""`bench.py` on the GPU: one JSON line carrying the keys the benchmark
contract names (value, roofline, cpu_baseline, e2e with its copy sizes,
clocks, the launch count), on the small simple-cubic workload."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_line_carries_the_contract_keys(tmp_path):
    env = dict(os.environ, JAMS_LLG_TUNE_CACHE=str(tmp_path / "tune.txt"))
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "sc32", "--steps", "20",
                          "--warmup", "3", "--no-accuracy", "--no-extra", "--ref-gpu", "off"],
                         capture_output=True, text=True, timeout=900, cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["value"] > 0 and d["steps"] == 20 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["unit"] == "spin-steps/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == "sc32" and d["config"]["spins"] == 32768
    # this library's launches: two stage kernels per Heun step, or one where
    # the autotuner picks the fused step
    assert d["gpu_launches"] in (d["steps"], 2 * d["steps"])
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["achieved"] > 0 and r["peak"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    assert r["kernel"].startswith(("tiled_stage<FamSC", "fused_heun<FamSC"))
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    e = d["e2e"]
    # the FP64 state each way, every step
    assert e["value"] > 0 and e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == 32768 * 3 * 8
    c = d["clocks"]
    assert "sm_mhz" in c and "sm_max_mhz" in c and isinstance(c["reasons"], list)
