"""bench.py's output contract, on CPU.

The reference arm (the CPU restatement of the reference's path) runs here at
the small 2,000 x 10,000 workload and must print exactly one JSON line with
the contract's keys; the GPU arm must fail loudly without a GPU rather than
fall back to the CPU."""
import json
import os
import subprocess
import sys

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args, timeout=300):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                          capture_output=True, text=True, timeout=timeout)


def test_reference_arm_prints_one_contract_line():
    out = _run("--impl", "reference", "--config", "c1", "--steps", "1", "--warmup", "1")
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in rec, key
    assert rec["impl"] == "reference" and rec["unit"] == "fits/hr" and rec["value"] > 0
    assert rec["higher_is_better"] is True and rec["steps"] == 1 and rec["warmup"] == 1
    assert rec["config"]["workload"] == "c1_n2000_m10000"
    cb = rec["cpu_baseline"]
    assert cb["value"] == rec["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]
    assert rec["e2e"]["value"] == rec["value"]
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["e2e"]["d2h_bytes_per_step"] == 0


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_gpu_arm_fails_without_a_gpu():
    out = _run("--steps", "1", "--warmup", "1")
    assert out.returncode != 0
    assert out.stdout.strip() == ""


def test_bench_helpers_pick_the_form_and_the_peak():
    """AUTO's per-width form, split-term counts and the peak the roofline
    divides by (sustained bf16 for the serving step's operator)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench._resolve("auto", 48) == "fp8x5" and bench._resolve("auto", 49) == "bf16x3"
    assert bench._resolve("fp16x2", 16) == "fp16x2"
    assert [bench._nsplit(p) for p in ("bf16x3", "fp8x5", "fp16x2", "fp32")] == [3, 5, 2, 0]
    hbm, burst, src_b = bench._peaks()
    _, sust, src_s = bench._peaks(sustained=True)
    assert hbm > 0 and burst >= sust > 0
    assert "sustained" in src_s or src_s == "fallback"
