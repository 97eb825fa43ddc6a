#!/usr/bin/env python
"""REML fits/hr on one GB300: the matrix-free REML hot path of COHERIT/GPU_REML.

Workload (default ``--config c2``): single-GRM REML, n=50,000 samples x
m=500,000 SNPs from the MAF~U(0.05,0.5)/HWE generator (synthetic; genotypes
generated on the device), phenotype with h2=0.3 from 5,000 causal SNPs,
10 N(0,1) covariates + intercept, 64 Rademacher SLQ probes (30-step
Lanczos), projected-core preconditioner.  A step is one complete REML fit
(operator applications, block PCG, SLQ, AI/NNLS line search).

Arms:
  ours       (default) the mixed-precision tensor-core form (BF16 genotypes,
             BF16x3 right-hand sides, FP32 PCG, FP64 small solves).  The same
             line reports the plain FP32 single-fit GPU form (CUDA-core FP32
             operator) as ``plain_fp32``, the operator roofline, and the CPU
             baseline (the oracle's FP32 restatement of kv_impl_streamed,
             timed on a bounded sample and scaled by the operator work the GPU
             fit performed).
  reference  ``--impl reference``: the CPU restatement of the reference path
             (the reference itself needs jax/numba, absent on these machines)
             on all host cores, on bounded samples of the same workload.

Timing: W warm-up fits, then K timed fits bracketed by barrier +
synchronize; inputs (6.25 GB of packed genotypes per copy) exceed the 129 MB
L2, so no explicit flush is needed.  ``value`` is device-timed with the
phenotype and covariates already resident; ``e2e`` times the public API call
with the phenotype/covariates copied from pinned host memory each step and
the variance components read back.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            pk = json.load(f)
        return float(pk.get("hbm_gbs", 6800.0)), float(pk.get("bf16_tflops", 1897.9)), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU port

def cpu_operator_sample(n: int, m_sample: int, k: int, seed: int, reps: int = 2):
    """Seconds per FP32 streamed application of the oracle port on m_sample SNPs."""
    from oracle import geno as og

    codes = og.synth_codes(seed, n, np.arange(m_sample))
    mean, inv, _ = og.stats(codes)
    W = m_sample
    packed = [og.pack_block(codes)]
    mbc = np.zeros((1, 4 * ((W + 3) // 4)), np.float32)
    ibc = np.zeros_like(mbc)
    mbc[0, :W] = mean
    ibc[0, :W] = inv
    V = np.random.default_rng(0).normal(size=(n, k)).astype(np.float32)
    og.kv_streamed_fp32(packed, [W], mbc, ibc, float(np.count_nonzero(inv > 0)), V)
    t0 = time.perf_counter()
    for _ in range(reps):
        og.kv_streamed_fp32(packed, [W], mbc, ibc, float(np.count_nonzero(inv > 0)), V)
    return (time.perf_counter() - t0) / reps


def cpu_fit_estimate(wl, apps: int, cols: int, budget_s: float = 20.0):
    """CPU seconds for one fit, scaled from two sampled application widths."""
    m_sample = 2048
    k1, k2 = 4, 64
    t1 = cpu_operator_sample(wl.n, m_sample, k1, wl.seed)
    t2 = cpu_operator_sample(wl.n, m_sample, k2, wl.seed)
    per_col = max((t2 - t1) / (k2 - k1), 0.0)
    fixed = max(t1 - per_col * k1, 0.0)
    scale = wl.m / m_sample
    t_fit = scale * (apps * fixed + cols * per_col)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    sample = (f"oracle FP32 kv_impl_streamed port, n={wl.n}, {m_sample}-SNP call block, "
              f"k={k1} and k={k2}; scaled by m/{m_sample} and by the fit's {apps} operator "
              f"applications / {cols} RHS columns")
    return t_fit, cores, sample


# ----------------------------------------------------------------- our arm

def build_problem(wl, device):
    import torch

    from coherit_gb300 import synth
    from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource

    st = GenoBlockStreamer(SyntheticSource(wl.n, wl.m, seed=wl.seed),
                           component_block_sizes=list(wl.components) if wl.components else None,
                           device=device, precision="bf16x3")
    y, X, _, _ = synth.phenotype(wl.seed, wl.n, wl.m, h2=wl.h2, n_causal=wl.n_causal,
                                 n_covar=wl.n_covar)
    return st, y, X


def make_fitter(st, wl, precision):
    from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter

    cfg = FitConfig(slq_samples=wl.slq_samples, slq_m=wl.slq_m, precond_rank=wl.precond_rank,
                    reml_pcg_tol=wl.pcg_tol, minq_iter=wl.minq_iter, max_pcg_iters=1000,
                    slq_mode="raw", precision=precision, sketch_precision="bf16x1",
                    cache_reml_setup=True, seed=wl.seed)
    return InfinitesimalREMLFitter(cfg, [st])


def operator_roofline(st, k, hbm_peak, reps=10):
    import torch

    from coherit_gb300 import _lib

    V = torch.randn(st.n, k, device=st.dev)
    for _ in range(3):
        st.kv(V)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        st.kv(V)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    alg_bytes = st.n * ((st.m + 3) // 4) + 8 * st.n * k + 8 * st.m
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "operator_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tr = json.load(f)
        key = f"{st.n}x{st.m}x{k}"
        traffic = tr.get(key)
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4), "traffic": traffic,
            "kernel": "genotype operator application (K1 + K2 + prep), k=%d" % k,
            "ms_per_application": round(ms, 4), "algorithmic_bytes": alg_bytes}


def run_ours(args, wl):
    import torch

    from coherit_gb300 import _lib

    ws, rank, local = _dist()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if ws > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl", device_id=dev)
        dist = tdist
    lib = _lib.load()
    hbm_peak, _, peak_src = _peaks()
    st, y, X = build_problem(wl, dev)
    fitter = make_fitter(st, wl, args.precision)
    y_pin = torch.as_tensor(y).pin_memory()
    X_pin = torch.as_tensor(X).pin_memory()
    y_dev = y_pin.to(dev)
    X_dev = X_pin.to(dev)
    h2s = []

    def one_fit(host: bool):
        if host:
            yd = y_pin.to(dev, non_blocking=True)
            Xd = X_pin.to(dev, non_blocking=True)
        else:
            yd, Xd = y_dev, X_dev
        res = fitter.fit_infinitesimal(yd, Xd)
        vc = np.asarray(res.var_components, dtype=np.float64)  # host copy of the result
        h2s.append(res.heritability)
        return res, vc

    for _ in range(args.warmup):
        one_fit(False)
    torch.cuda.synchronize()
    apps0, cols0 = st.op_stats["apps"], st.op_stats["cols"]
    launches0 = lib.coherit_launch_count()
    sampler = ClockSampler(local)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    lat = []
    e0.record(stream)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        one_fit(False)
        lat.append(time.perf_counter() - t0)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    dev_s = e0.elapsed_time(e1) / 1e3
    launches = lib.coherit_launch_count() - launches0
    apps = (st.op_stats["apps"] - apps0) / args.steps
    cols = (st.op_stats["cols"] - cols0) / args.steps
    # end to end through the public API with host inputs
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_fit(True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([dev_s, e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s, e2e_s = float(t[0]), float(t[1])
    total_fits = args.steps * ws
    value = total_fits / (dev_s / 3600.0)
    e2e_val = total_fits / (e2e_s / 3600.0)
    result = None
    if rank == 0:
        roof = operator_roofline(st, wl.n_covar + 2, hbm_peak)
        roof["peak_source"] = peak_src
        plain = None
        if not args.no_plain:
            pf = make_fitter(st, wl, "fp32")
            t0 = time.perf_counter()
            pres = pf.fit_infinitesimal(y_dev, X_dev)
            torch.cuda.synchronize()
            tp = time.perf_counter() - t0
            plain = {"fits_per_hr": round(3600.0 / tp, 3), "fit_s": round(tp, 3),
                     "h2": round(pres.heritability, 6),
                     "abs_dh2_vs_mixed": round(abs(pres.heritability - h2s[-1]), 6)}
        cpu = None
        if not args.no_cpu:
            t_fit, cores, sample = cpu_fit_estimate(wl, apps, cols)
            cpu = {"value": round(3600.0 / t_fit, 4), "unit": "fits/hr", "cores": cores,
                   "kind": "port", "sample": sample, "fit_s_extrapolated": round(t_fit, 1)}
        lat_sorted = sorted(lat)
        result = {
            "metric": "REML fits/hr (mixed-precision BF16x3 tensor-core form; plain FP32 form and p50/p99 fit latency alongside)",
            "value": round(value, 3),
            "unit": "fits/hr",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(dev_s / args.steps * 1e3, 2),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "bf16x3 genotype operator, fp32 PCG, fp64 small solves",
            "data": "synthetic (device-generated MAF~U(0.05,0.5) HWE genotypes; phenotype h2=%.2f)" % wl.h2,
            "config": {"workload": wl.name, "n": wl.n, "m": wl.m, "slq_probes": wl.slq_samples,
                       "lanczos_steps": wl.slq_m, "covariates": wl.n_covar,
                       "precond_rank": wl.precond_rank, "pcg_tol": wl.pcg_tol,
                       "parallelism": f"replicas x{ws}",
                       "l2_policy": "inputs larger than L2 (2 x 6.25 GB packed genotypes)"},
            "latency_s": {"p50": round(statistics.median(lat), 3),
                          "p99": round(lat_sorted[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)], 3)},
            "h2": round(h2s[-1], 6),
            "operator_apps_per_fit": apps,
            "rhs_columns_per_fit": cols,
            "e2e": {"value": round(e2e_val, 3), "unit": "fits/hr",
                    "h2d_bytes_per_step": int(y_pin.numel() * 4 + X_pin.numel() * 4),
                    "d2h_bytes_per_step": 8 * 2},
            "gpu_launches": int(launches),
            "roofline": roof,
            "plain_fp32": plain,
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
    st.close()
    if dist is not None:
        dist.destroy_process_group()
    return result


def run_reference(args, wl):
    ws, rank, _ = _dist()
    if rank != 0:
        return None
    # The reference (jax + numba) is not installable here; its CPU path is
    # restated by the oracle.  Each step times one bounded sample: one FP32
    # streamed application of a 2048-SNP call block at n on all host cores,
    # scaled to a whole fit by the operator work a fit performs.
    apps, cols = args.ref_apps, args.ref_cols
    for _ in range(args.warmup):
        cpu_operator_sample(wl.n, 2048, 16, wl.seed, reps=1)
    times = []
    for _ in range(args.steps):
        t_fit, cores, sample = cpu_fit_estimate(wl, apps, cols)
        times.append(t_fit)
    t_fit = statistics.median(times)
    value = 3600.0 / t_fit
    return {
        "impl": "reference",
        "metric": "REML fits/hr (mixed-precision BF16x3 tensor-core form; plain FP32 form and p50/p99 fit latency alongside)",
        "value": round(value, 5),
        "unit": "fits/hr",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 (reference arithmetic)",
        "data": "synthetic",
        "config": {"workload": wl.name, "n": wl.n, "m": wl.m},
        "cpu_baseline": {"value": round(value, 5), "unit": "fits/hr", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 5), "unit": "fits/hr", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c2")
    ap.add_argument("--precision", default="bf16x3")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-apps", type=float, default=200.0,
                    help="operator applications per fit assumed by the reference arm")
    ap.add_argument("--ref-cols", type=float, default=4000.0,
                    help="right-hand-side columns per fit assumed by the reference arm")
    args = ap.parse_args()
    from coherit_gb300.configs import WORKLOADS

    wl = WORKLOADS[args.config]
    out = run_reference(args, wl) if args.impl == "reference" else run_ours(args, wl)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
