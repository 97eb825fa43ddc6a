#!/usr/bin/env python
"""REML fits/hr on one GB300: the matrix-free REML hot path of COHERIT/GPU_REML.

Workload (default ``--config c2``): single-GRM REML, n=50,000 samples x
m=500,000 SNPs from the MAF~U(0.05,0.5)/HWE generator (synthetic; genotypes
generated on the device); each phenotype has h2=0.3 from 5,000 causal SNPs,
10 N(0,1) covariates + intercept; 64 Rademacher SLQ probes, 30-step Lanczos,
PCG tol 1e-5.  A step is one serving batch: R (``--requests``, default 8)
phenotypes submitted together to the REMLServer, each fitted completely
(operator applications, block PCG, affine SLQ, AI/NNLS line search), their
operator applications batched into shared launches.

Arms:
  ours       (default) the mixed-precision batched serving form (BF16
             genotypes, BF16x3 right-hand sides, FP32 PCG, FP64 small
             solves).  The same line reports the same fits run one at a time
             through the single-fit model API (``single_fit_mixed``), the
             plain FP32 single-fit GPU form (CUDA-core FP32 operator,
             ``plain_fp32_single_fit``), the operator roofline at the batched
             width, and the CPU baseline (the oracle's FP32 restatement of
             kv_impl_streamed, timed on a bounded sample and scaled by the
             operator work of one fit).  ``sparse12`` times the rare-variant
             operator (per-SNP entry lists, MAF~U(0.0005,0.01)) at the same
             n x m and width as the roofline.
  reference  ``--impl reference``: the CPU restatement of the reference path
             (the reference itself needs jax/numba, absent on these machines)
             on all host cores, on bounded samples of the same workload.

Timing: W warm-up steps, then K timed steps bracketed by barrier +
synchronize; inputs (6.25 GB of packed genotypes per copy) exceed the 129 MB
L2, so no explicit flush is needed.  ``value`` is device-timed with the
phenotypes and covariates already resident; ``e2e`` times the same serving
steps through the public API with phenotypes/covariates taken from pinned
host memory and the variance components returned to the host.
"""
from __future__ import annotations

import argparse
import collections
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


def replica_totals(dev_s: float, e2e_s: float, steps: int, requests: int, dist=None,
                   device="cpu"):
    """Whole-job fits/hr of N independent replicas (one per rank, no
    data-path collective): every rank served steps x requests fits and the
    job took as long as its slowest rank (MAX over ranks of both times).
    Returns (device s, end-to-end s, value, e2e value)."""
    import torch

    ws = 1
    if dist is not None:
        t = torch.tensor([dev_s, e2e_s], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s, e2e_s = float(t[0]), float(t[1])
        ws = dist.get_world_size()
    total = steps * requests * ws
    return dev_s, e2e_s, total / (dev_s / 3600.0), total / (e2e_s / 3600.0)


def _peaks(sustained: bool = False):
    """(HBM GB/s, bf16 TFLOP/s, source): the measured copy bandwidth and the
    burst cuBLAS bf16 rate, or with ``sustained`` the rate of a seconds-long
    GEMM loop under the power cap -- the denominator for a kernel that runs
    inside a long step (the operator in a serving step runs back to back for
    seconds at the power cap, as the sustained GEMM does)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            pk = json.load(f)
        ten = float(pk.get("bf16_tflops_sustained" if sustained else "bf16_tflops",
                           pk.get("bf16_tflops", 1897.9)))
        return (float(pk.get("hbm_gbs", 6800.0)), ten,
                "measured (sustained bf16)" if sustained else "measured (burst bf16)")
    return 6800.0, 1700.0 if sustained else 1900.0, "fallback"


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
        sm, smax, power, reasons = [], [], [], set()
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
                try:
                    power.append(float(parts[3].split()[0]))
                except (ValueError, IndexError):
                    pass
                for name, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "sm_mhz_min": min(sm) if sm else None,
                "power_w_median": statistics.median(power) if power else None,
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


def _cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def cpu_vector_sample(n: int, k: int, reps: int = 3):
    """Seconds of the block-PCG vector work of one iteration (state and
    direction updates, column reductions) of the oracle port on (n, k)."""
    from oracle import pcg as opcg

    rng = np.random.default_rng(0)
    X, R, P, AP, Z = (rng.normal(size=(n, k)).astype(np.float32) for _ in range(5))
    rs = np.einsum("ij,ij->j", R, Z).astype(np.float64)
    active = np.ones(k, dtype=bool)
    t0 = time.perf_counter()
    for _ in range(reps):
        opcg._state_update(X, R, P, rs, AP, active)
        opcg._direction_update(P, R, Z, rs, 1e-30)
    return (time.perf_counter() - t0) / reps


def cpu_fit_estimate(wl, apps: float, cols: float, budget_s: float = 20.0):
    """CPU seconds for one fit at the workload's size, extrapolated: the
    oracle's FP32 kv_impl_streamed port timed on a 1,024-SNP call block at n
    samples for two widths (a fixed and a per-column cost), scaled by
    m / 1,024 and by the fit's operator applications and right-hand-side
    columns (counted on the GPU in the same run), plus the PCG vector work
    of one iteration per application."""
    m_sample = 1024
    k1, k2 = 4, 64
    t1 = cpu_operator_sample(wl.n, m_sample, k1, wl.seed)
    t2 = cpu_operator_sample(wl.n, m_sample, k2, wl.seed)
    per_col = max((t2 - t1) / (k2 - k1), 0.0)
    fixed = max(t1 - per_col * k1, 0.0)
    scale = wl.m / m_sample
    k_typ = max(1, int(round(cols / max(apps, 1.0))))
    t_vec = cpu_vector_sample(wl.n, k_typ)
    t_fit = scale * (apps * fixed + cols * per_col) + apps * t_vec
    sample = (f"extrapolated: oracle FP32 kv_impl_streamed port, n={wl.n}, {m_sample}-SNP call "
              f"block at k={k1} and k={k2}, scaled by m/{m_sample} and by {apps:.1f} operator "
              f"applications / {cols:.1f} RHS columns per fit, plus PCG vector work at k={k_typ} "
              f"per application")
    return t_fit, _cores(), sample


def cpu_c1_fit():
    """One whole fit of the small CPU-runnable configuration by the CPU port
    of the reference path, timed end to end on all host cores: per-call
    packed genotypes (4,096-SNP calls) applied by the FP32 kv_impl_streamed
    restatement, the affine SLQ cache (30 probes, 30 Lanczos steps), the
    oracle's block PCG (tol 1e-6) and AI-REML driver.  Returns (seconds,
    h2)."""
    from coherit_gb300 import synth
    from coherit_gb300.configs import C1
    from oracle import geno as og
    from oracle import reml as oreml
    from oracle import slq as oslq

    n, m = C1.n, C1.m
    codes = og.synth_codes(C1.seed, n, np.arange(m))
    y, X, _, _ = synth.phenotype(C1.seed, n, m, h2=C1.h2, n_causal=C1.n_causal,
                                 n_covar=C1.n_covar, noise_var=0.5)
    probes = np.random.default_rng(C1.seed).choice([-1.0, 1.0], size=(n, C1.slq_samples))
    t0 = time.perf_counter()
    starts, widths, _, _ = og.call_geometry(m, 4096)
    W = 4 * ((int(widths.max()) + 3) // 4)
    packed = [og.pack_block(codes[:, s0:s0 + w]) for s0, w in zip(starts, widths)]
    mean, inv, cnt = og.stats(codes)
    mbc = np.zeros((len(widths), W), np.float32)
    ibc = np.zeros_like(mbc)
    for c, (s0, w) in enumerate(zip(starts, widths)):
        mbc[c, :w] = mean[s0:s0 + w]
        ibc[c, :w] = inv[s0:s0 + w]
    eff = float(np.count_nonzero(inv > 0))
    _, _, _, atom = og.stats_summary(cnt, *og.raw_counts(codes)[1:], mean, inv, n)

    def K(V):
        return og.kv_streamed_fp32(packed, widths, mbc, ibc, eff, V)

    yo, _, _ = oreml.standardize(y)
    cache = oslq.affine_cache(K, n, probes, C1.slq_m)
    ctx = oreml.Context(yo, [K], X, diag_atoms=[atom], affine_cache=cache, pcg_tol=C1.pcg_tol,
                        maxiter=1000)
    po, _, _ = oreml.fit(ctx, minq_iter=C1.minq_iter)
    t = time.perf_counter() - t0
    return t, oreml.heritability(po, 1, [atom])


# ----------------------------------------------------------------- our arm

def build_problem(wl, device):
    from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource

    return GenoBlockStreamer(SyntheticSource(wl.n, wl.m, seed=wl.seed),
                             component_block_sizes=list(wl.components) if wl.components else None,
                             device=device, precision="bf16x3")


def make_phenotypes(st, wl, R: int, seed: int):
    """R phenotypes over the resident genotypes: for each, wl.n_causal causal
    SNPs with N(0,1) effects on standardised genotypes (one Z B product on the
    device for all R), scaled to variance wl.h2, plus N(0, 1 - wl.h2) noise;
    covariates [1, wl.n_covar x N(0,1)].  Returns device tensors."""
    import torch

    rng = np.random.default_rng(seed)
    B = np.zeros((st.m, R), dtype=np.float32)
    for r in range(R):
        causal = rng.choice(st.m, size=min(wl.n_causal, st.m), replace=False)
        B[causal, r] = rng.normal(size=causal.size)
    g = st.zxb(torch.as_tensor(B, device=st.dev)).double()
    g = g * torch.sqrt(wl.h2 / g.var(dim=0, unbiased=False))
    gen = torch.Generator(device=st.dev).manual_seed(seed)
    noise = torch.randn((st.n, R), generator=gen, device=st.dev, dtype=torch.float64)
    ys = (g + noise * math.sqrt(1.0 - wl.h2)).float()
    Xs = []
    for r in range(R):
        X = torch.randn((st.n, wl.n_covar + 1), generator=gen, device=st.dev)
        X[:, 0] = 1.0
        Xs.append(X)
    return [ys[:, r].contiguous() for r in range(R)], Xs


def fit_kwargs(wl):
    return dict(n_rand_vec=30, maxiter=1000, minq_iter=wl.minq_iter, slq_samples=wl.slq_samples,
                slq_m=wl.slq_m, pcg_tol=wl.pcg_tol, verbose=False, seed=wl.seed)


def make_fitter(st, wl, precision, slq_workspace_bytes=None):
    from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter

    cfg = FitConfig(slq_samples=wl.slq_samples, slq_m=wl.slq_m, precond_rank=wl.precond_rank,
                    reml_pcg_tol=wl.pcg_tol, minq_iter=wl.minq_iter, max_pcg_iters=1000,
                    slq_mode="raw", precision=precision, sketch_precision="bf16x1",
                    cache_reml_setup=True, seed=wl.seed, verbose=False,
                    slq_workspace_bytes=slq_workspace_bytes)
    return InfinitesimalREMLFitter(cfg, [st])


def _percentile(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, max(0, int(math.ceil(q * len(xs))) - 1))]


def _nsplit(precision: str) -> int:
    return {"bf16x3": 3, "bf16x2": 2, "fp16x2": 2, "bf16x1": 1, "fp8x5": 5}.get(precision, 0)


def _resolve(precision: str, k: int) -> str:
    """The form AUTO takes at width k: E4M3 tiles up to 48 columns, bf16x3 above."""
    if precision == "auto":
        return "fp8x5" if k <= 48 else "bf16x3"
    return precision


def operator_roofline(st, k, hbm_peak, tensor_peak, reps=10, precision=None):
    """Device time of one operator application at width k, its HBM and
    tensor fractions (algorithmic bytes n*ceil(m/4) + 8nk + 8m and flops
    4nmk), timed with CUDA events on the launching stream.  For the
    tensor-core precisions also the MMA instruction count of the two
    contractions (M = 128, K = 16 for the 16-bit forms and 32 for E4M3:
    2 * n_pad * m_pad / (128 K) per launch) and the SM cycles per
    instruction this time implies: one issuing thread pays a fixed 120
    cycles per instruction up to N = 224 on GB300 (bench.py --mma-rate), so
    narrow launches are bound by the instruction count, not by HBM."""
    import torch

    precision = precision or st.precision
    V = torch.randn(st.n, k, device=st.dev)
    for _ in range(3):
        st.kv(V, precision=precision)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        st.kv(V, precision=precision)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    alg_bytes = st.n * ((st.m + 3) // 4) + 8 * st.n * k + 8 * st.m
    alg_flops = 4.0 * st.n * st.m * k
    gbs = alg_bytes / (ms * 1e-3) / 1e9
    tfs = alg_flops / (ms * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "operator_traffic.json")
    if os.path.exists(tpath):
        kp = (k + 15) // 16 * 16
        with open(tpath) as f:
            traffic = json.load(f).get(f"{st.n}x{st.m}x{kp}")
    hbm_frac, ten_frac = gbs / hbm_peak, tfs / tensor_peak
    if ten_frac >= hbm_frac:
        roof = {"bound": "tensor", "achieved": round(tfs, 1), "peak": tensor_peak,
                "unit": "TFLOP/s", "frac": round(ten_frac, 4)}
    else:
        roof = {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(hbm_frac, 4)}
    roof.update({"traffic": traffic,
                 "kernel": f"genotype operator application (prep + K1 + K2), k={k}, {precision}",
                 "ms_per_application": round(ms, 4), "algorithmic_bytes": alg_bytes,
                 "algorithmic_flops": alg_flops, "hbm_gbs": round(gbs, 1),
                 "hbm_frac": round(hbm_frac, 4), "tensor_tflops": round(tfs, 1),
                 "tensor_frac": round(ten_frac, 4)})
    form = _resolve(precision, k)
    ns = _nsplit(form)
    if ns:
        info = st.info()
        kp = (k + 15) // 16 * 16
        max_cols = 128 if form == "fp16x2" else (256 // ns) // 16 * 16
        launches = -(-kp // max_cols)
        kk = 32 if form == "fp8x5" else 16
        instr = 2.0 * info["n_pad"] * info["m_pad"] / (128.0 * kk) * launches
        sm_hz, sms = _sm_clock_hz(), torch.cuda.get_device_properties(st.dev).multi_processor_count
        n_instr = ns * min(kp, max_cols)
        # Dense work the instructions execute (every split term, padding
        # columns included) against the nominal dense rate of their operand
        # type: 2.25 PFLOP/s for 16-bit operands, 4.5 for E4M3.
        executed = instr * 2.0 * 128 * n_instr * kk / (ms * 1e-3) / 1e12
        nominal = 4500.0 if form == "fp8x5" else 2250.0
        roof["mma_issue"] = {
            "instructions_per_application": int(instr),
            "form": form, "k_per_instruction": kk,
            "n_per_instruction": n_instr,
            "cycles_per_instruction_per_sm": round(ms * 1e-3 * sm_hz * sms / instr, 1),
            "sm_clock_mhz_assumed": sm_hz / 1e6,
            "executed_tflops": round(executed, 1),
            "nominal_dense_tflops": nominal,
            "executed_frac_of_nominal": round(executed / nominal, 3)}
    return roof


def _sm_clock_hz() -> float:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f).get("sm_max_mhz", 2070.0)) * 1e6
    return 2070e6


def sparse12_operator(n, m, k, hbm_peak, dense_ms, seed, reps=10):
    """The rare-variant (sparse12) operator at the headline shape: n samples x
    m SNPs with MAF ~ U(0.0005, 0.01) held as per-SNP entry lists in HBM
    (built on the device by the generator), K V and Z^T V at width k timed
    with CUDA events on the launching stream.  Algorithmic bytes of K V:
    4 per stored entry + 16 per SNP (offsets, mean, inv) + 8nk (V read, out
    written); the gathers / scatter-adds of 2 x 4k bytes per entry run out of
    L2 (V and out are L2-resident), so the L2 rate is reported beside the HBM
    fraction."""
    import torch

    from coherit_gb300.sparse_stream import SparseGenoBlockStreamer, SyntheticRareSource

    t0 = time.perf_counter()
    sp = SparseGenoBlockStreamer(SyntheticRareSource(n, m, seed=seed, maf_range=(0.0005, 0.01)))
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    nnz = sp.info()["nnz"]
    V = torch.randn(n, k, device=sp.dev)
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    kv_ms = timed(lambda: sp.kv(V))
    xtv_ms = timed(lambda: sp.xtv(V))
    alg = 4 * nnz + 16 * m + 8 * n * k
    gbs = alg / (kv_ms * 1e-3) / 1e9
    l2_tbs = 2 * 4 * nnz * k / (kv_ms * 1e-3) / 1e12
    sp.close()
    return {"workload": f"n{n}_m{m}_rare_maf0.0005-0.01", "n": n, "m": m, "entries": nnz,
            "k": k, "build_s": round(build_s, 3), "kv_ms": round(kv_ms, 3),
            "xtv_ms": round(xtv_ms, 3), "dense_kv_ms_same_shape": round(dense_ms, 3),
            "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(gbs / hbm_peak, 4), "traffic": None,
                         "kernel": "sparse K V (prep + fused gather/scatter + finish)",
                         "algorithmic_bytes": alg, "l2_gather_scatter_TBps": round(l2_tbs, 2)}}


def serve_step(srv, ys, Xs, host: bool):
    """One step: all R requests submitted at once; returns their results."""
    if host:
        futs = [srv.submit(y.cpu().numpy(), X.cpu().numpy()) for y, X in zip(ys, Xs)]
    else:
        futs = [srv.submit(y, X) for y, X in zip(ys, Xs)]
    return [f.result() for f in futs]


def serving_stream(st, wl, n_requests: int, rate_per_s: float, seed: int, max_active: int,
                   min_subset: int | None = None, precision: str = "bf16x3",
                   precond_rank: int = 0):
    """A bounded stream of heterogeneous requests with Poisson arrivals over
    the resident genotypes (the serving workload's request mix on this
    matrix): each request a random sample subset (size log-uniform in
    [min_subset, n], default n/5), 1-20 N(0,1) covariates + intercept,
    h2 ~ U(0.05, 0.8) from wl.n_causal causal SNPs.  Requests arrive while
    earlier ones are on the GPU and join their batched launches.  Returns the
    stream's summary."""
    import torch

    from coherit_gb300.serving import REMLServer

    rng = np.random.default_rng(seed)
    n = st.n
    B = np.zeros((st.m, n_requests), dtype=np.float32)
    for r in range(n_requests):
        causal = rng.choice(st.m, size=min(wl.n_causal, st.m), replace=False)
        B[causal, r] = rng.normal(size=causal.size)
    G = st.zxb(torch.as_tensor(B, device=st.dev)).double().cpu().numpy()
    reqs = []
    for r in range(n_requests):
        lo = float(min_subset) if min_subset else n / 5
        size = int(np.exp(rng.uniform(np.log(lo), np.log(n))))
        mask = np.zeros(n, dtype=bool)
        mask[rng.choice(n, size=size, replace=False)] = True
        h2 = rng.uniform(0.05, 0.8)
        g = G[mask, r]
        g = g * np.sqrt(h2 / g.var())
        y = (g + rng.normal(scale=np.sqrt(1 - h2), size=size)).astype(np.float32)
        p = int(rng.integers(1, 21))
        X = np.column_stack([np.ones(size), rng.normal(size=(size, p))]).astype(np.float32)
        reqs.append((y, X, mask))
    gaps = rng.exponential(1.0 / rate_per_s, size=n_requests)
    srv = REMLServer(st, max_active=max_active, precision=precision, fit_kwargs=fit_kwargs(wl),
                     precond_rank=precond_rank)
    b0, c0 = srv.batcher.launches, srv.batcher.columns
    t0 = time.perf_counter()
    futs = []
    for (y, X, mask), gap in zip(reqs, gaps):
        time.sleep(float(gap))
        futs.append(srv.submit(y, X, sample_mask=mask))
    res, failed = [], []
    try:
        for i, f in enumerate(futs):
            try:
                res.append(f.result())
            except Exception as err:  # a failed fit is reported, not fatal
                failed.append(f"request {i}: {type(err).__name__}: {str(err)[:200]}")
        wall = time.perf_counter() - t0
        per_launch = list(srv.batcher.requests_per_launch)
        launches = srv.batcher.launches - b0
        columns = srv.batcher.columns - c0
    finally:
        srv.close()
    lat = [r.latency for r in res] or [float("nan")]
    return {"requests": n_requests, "completed": len(res), "failed": failed,
            "arrival_rate_per_s": round(rate_per_s, 3),
            "fits_per_hr": round(len(res) / (wall / 3600.0), 1),
            "latency_s": {"p50": round(statistics.median(lat), 3),
                          "p99": round(_percentile(lat, 0.99), 3)},
            "subset_sizes": [int(m.sum()) for _, _, m in reqs][:8],
            "operator_launches": launches,
            "operator_launches_per_fit": round(launches / max(len(res), 1), 1),
            "rhs_columns_per_launch": round(columns / max(launches, 1), 1),
            "mean_requests_per_launch": round(float(np.mean(per_launch)), 2) if per_launch else 0.0,
            "max_active": max_active, "precision": precision, "precond_rank": precond_rank,
            "seed": seed}


def run_ours(args, wl):
    import torch

    from coherit_gb300 import _lib
    from coherit_gb300.serving import REMLServer

    ws, rank, local = _dist()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if ws > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl", device_id=dev)
        dist = tdist
    lib = _lib.load()
    hbm_peak, tensor_peak, peak_src = _peaks(sustained=True)
    st = build_problem(wl, dev)
    R = args.requests
    ys, Xs = make_phenotypes(st, wl, R, seed=wl.seed + 17 * rank)
    # Host copies for the end-to-end leg (pinned, as a serving front end holds them).
    ys_host = [y.cpu().pin_memory() for y in ys]
    Xs_host = [X.cpu().pin_memory() for X in Xs]
    tuner = None
    if not args.no_autotune:
        # Launch configurations of the widths the batcher issues (16-column
        # steps up to its cap), tuned on these genotypes before warm-up.
        from coherit_gb300.serving import _MAX_BATCH_COLS

        widths = list(range(16, _MAX_BATCH_COLS.get(args.precision, 80) + 1, 16))
        tuner = st.autotune(widths, precision=args.precision, reps=1)
    srv = REMLServer(st, max_active=R, precision=args.precision, fit_kwargs=fit_kwargs(wl),
                     batch_window_s=args.batch_window)

    cold_fit_s = None
    for w in range(args.warmup):
        t0 = time.perf_counter()
        serve_step(srv, ys, Xs, host=False)
        torch.cuda.synchronize()
        if w == 0:
            # The first batch builds the shared SLQ cache and preconditioner set-up.
            cold_fit_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    launches0 = lib.coherit_launch_count()
    b0, c0 = srv.batcher.launches, srv.batcher.columns
    n_res0 = len(srv.results)
    sampler = ClockSampler(local)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # The timed region is also the profiler's capture range
    # (ncu --profile-from-start off); without a profiler these are no-ops.
    torch.cuda.profiler.start()
    e0.record(stream)
    timed = []
    for _ in range(args.steps):
        timed.extend(serve_step(srv, ys, Xs, host=False))
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    dev_s = e0.elapsed_time(e1) / 1e3
    launches = lib.coherit_launch_count() - launches0
    op_launches = srv.batcher.launches - b0
    op_cols = srv.batcher.columns - c0
    # Device time of the batched operator launches inside the timed steps
    # (their own CUDA events): the rest of the step is solver work and idle.
    op_dev_ms = srv.batcher.device_ms(b0)
    timed_widths = list(srv.batcher.launch_widths[-op_launches:]) if op_launches else []
    # Operator applications the timed fits requested (a launch serves one
    # application of each request it carries).
    op_apps = float(sum(srv.batcher.requests_per_launch[b0:b0 + op_launches]))
    lat = [r.latency for r in timed]

    # End to end through the public API: phenotypes/covariates from pinned
    # host memory each step, variance components back on the host.
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        futs = [srv.submit(y.numpy(), X.numpy()) for y, X in zip(ys_host, Xs_host)]
        e2e_res = [f.result() for f in futs]
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    srv.close()
    dev_s, e2e_s, value, e2e_val = replica_totals(dev_s, e2e_s, args.steps, R, dist, dev)
    result = None
    if rank == 0:
        n_fits = args.steps * R
        fit_apps, fit_cols = op_apps / n_fits, op_cols / n_fits
        # The roofline is taken at the most frequent launch width (columns
        # rounded up to 16, as the launch pads them; the wider on a tie):
        # AUTO switches from E4M3 to bf16x3 tiles above 48 columns, so the
        # mean width would measure a form most launches do not use.
        widths = collections.Counter(-(-w // 16) * 16 for w in timed_widths)
        k_typ = (max(widths.items(), key=lambda kv: (kv[1], kv[0]))[0] if widths
                 else max(16, int(round(op_cols / max(op_launches, 1)))))
        launch_width_counts = {int(w): int(c) for w, c in sorted(widths.items())}
        roof = operator_roofline(st, k_typ, hbm_peak, tensor_peak, precision=args.precision)
        roof["peak_source"] = peak_src
        single = None
        plain = None
        if not args.no_single:
            # The same fits one at a time through the single-fit model API
            # (mixed precision, projected-core preconditioner, shared setup).
            fitter = make_fitter(st, wl, args.precision)
            fitter.fit_infinitesimal(ys[0], Xs[0])
            torch.cuda.synchronize()
            a0, k0 = st.op_stats["apps"], st.op_stats["cols"]
            t0 = time.perf_counter()
            sh2 = []
            for r in range(min(R, args.single_fits)):
                sh2.append(fitter.fit_infinitesimal(ys[r], Xs[r]).heritability)
            torch.cuda.synchronize()
            ts = (time.perf_counter() - t0) / len(sh2)
            single = {"fits_per_hr": round(3600.0 / ts, 3), "fit_s": round(ts, 4),
                      "operator_apps_per_fit": (st.op_stats["apps"] - a0) / len(sh2),
                      "rhs_columns_per_fit": (st.op_stats["cols"] - k0) / len(sh2),
                      "max_abs_dh2_vs_served": round(max(
                          abs(a - b.heritability) for a, b in zip(sh2, timed)), 6)}
        if not args.no_plain:
            # Plain FP32 single-fit form, warm (its shared setup built by a
            # first fit), timed on the second phenotype.
            pf = make_fitter(st, wl, "fp32")
            pf.fit_infinitesimal(ys[0], Xs[0])
            torch.cuda.synchronize()
            a0, k0 = st.op_stats["apps"], st.op_stats["cols"]
            t0 = time.perf_counter()
            pres = pf.fit_infinitesimal(ys[1 % R], Xs[1 % R])
            torch.cuda.synchronize()
            tp = time.perf_counter() - t0
            papps = st.op_stats["apps"] - a0
            pcols = st.op_stats["cols"] - k0
            pk = max(1, int(round(pcols / max(papps, 1))))
            plain = {"fits_per_hr": round(3600.0 / tp, 3), "fit_s": round(tp, 3),
                     "h2": round(pres.heritability, 6),
                     "abs_dh2_vs_served": round(
                         abs(pres.heritability - timed[1 % R].heritability), 6),
                     "operator_apps_per_fit": papps, "rhs_columns_per_fit": pcols,
                     "roofline": operator_roofline(st, pk, hbm_peak, tensor_peak,
                                                   precision="fp32", reps=3)}
        stream = None
        if args.stream > 0:
            stream = serving_stream(st, wl, args.stream, args.stream_rate, seed=wl.seed + 99,
                                    max_active=R, precision=args.precision,
                                    precond_rank=args.stream_precond)
        sparse = None
        if args.sparse12:
            sparse = sparse12_operator(wl.n, wl.m, k_typ, hbm_peak, roof["ms_per_application"],
                                       seed=wl.seed + 7)
        cpu = None
        if not args.no_cpu:
            c1_s, c1_h2 = cpu_c1_fit()
            t_fit, cores, sample = cpu_fit_estimate(wl, fit_apps, fit_cols)
            cpu = {"value": round(3600.0 / t_fit, 5), "unit": "fits/hr", "cores": cores,
                   "kind": "port", "extrapolated": True, "sample": sample,
                   "fit_s_extrapolated": round(t_fit, 1),
                   "c1_whole_fit": {"fit_s": round(c1_s, 2),
                                    "fits_per_hr": round(3600.0 / c1_s, 2),
                                    "h2": round(c1_h2, 6), "cores": cores,
                                    "workload": "c1_n2000_m10000 (measured end to end)"}}
        result = {
            "metric": METRIC,
            "value": round(value, 3),
            "unit": "fits/hr",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(dev_s / args.steps * 1e3, 2),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": f"{args.precision} genotype operator, fp32 PCG, fp64 small solves",
            "data": "synthetic (device-generated MAF~U(0.05,0.5) HWE genotypes; "
                    f"{R} phenotypes with h2={wl.h2}, {wl.n_causal} causal SNPs each)",
            "config": {"workload": wl.name, "n": wl.n, "m": wl.m,
                       "requests_per_step": R, "slq_probes": wl.slq_samples,
                       "lanczos_steps": wl.slq_m, "covariates": wl.n_covar,
                       "pcg_tol": wl.pcg_tol, "parallelism": f"replicas x{ws}",
                       "slq_cache": "the affine SLQ cache (slq_probes x lanczos_steps operator "
                                    "columns) is built once during warm-up and shared by every "
                                    "fit on these genotypes, as the reference's REMLProbeCache "
                                    "allows; each step re-fits the same R phenotypes",
                       "l2_policy": "inputs larger than L2 (2 x n*m/4 bytes of packed "
                                    "genotypes, 50 GB at n=100k, m=1M)"},
            "latency_s": {"p50": round(statistics.median(lat), 3),
                          "p99": round(_percentile(lat, 0.99), 3)},
            "cold_step_s": None if cold_fit_s is None else round(cold_fit_s, 3),
            "h2": [round(r.heritability, 4) for r in timed[:R]],
            "operator_launches_per_step": op_launches / args.steps,
            "operator_device_ms_per_step": round(op_dev_ms / args.steps, 1),
            "operator_share_of_step": round(op_dev_ms / (dev_s * 1e3), 3),
            "rhs_columns_per_launch": round(op_cols / max(op_launches, 1), 1),
            "launch_width_counts": launch_width_counts,
            "operator_apps_per_fit": round(fit_apps, 2),
            "rhs_columns_per_fit": round(fit_cols, 1),
            "e2e": {"value": round(e2e_val, 3), "unit": "fits/hr",
                    "h2d_bytes_per_step": int(sum(y.numel() * 4 + X.numel() * 4
                                                  for y, X in zip(ys_host, Xs_host))),
                    "d2h_bytes_per_step": int(sum(r.var_components.size * 8 for r in e2e_res))},
            "gpu_launches": int(launches),
            "roofline": roof,
            "autotune": tuner,
            "serving_stream": stream,
            "single_fit_mixed": single,
            "plain_fp32_single_fit": plain,
            "sparse12": sparse,
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
        if args.write_counts:
            with open(args.write_counts, "w") as f:
                json.dump({"workload": wl.name, "operator_apps_per_fit": fit_apps,
                           "rhs_columns_per_fit": fit_cols,
                           "source": "bench.py serving run (timed fits)"}, f, indent=1)
    st.close()
    if result is not None and args.c4_stream > 0:
        result["serving_stream_c4"] = c4_stream(args, dev)
    if dist is not None:
        dist.destroy_process_group()
    return result


def c4_stream(args, dev):
    """The c4 serving workload, bounded: ``--c4-stream`` requests (of c4's
    512) over one resident n=200,000 x m=600,000 matrix, sample subsets
    log-uniform in [1e4, 2e5], 1-20 covariates, h2 ~ U(0.05, 0.8), Poisson
    arrivals at ``--c4-rate`` per second, 8 fits in flight.  Runs after the
    headline workload's matrix is released."""
    import torch

    from coherit_gb300.configs import C4, C4_SUBSET_MIN
    from coherit_gb300.serving import _MAX_BATCH_COLS

    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    st = build_problem(C4, dev)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    try:
        if not args.no_autotune:
            st.autotune(list(range(16, _MAX_BATCH_COLS.get(args.precision, 80) + 1, 16)),
                        precision=args.precision, reps=1)
        out = serving_stream(st, C4, args.c4_stream, args.c4_rate, seed=C4.seed + 99,
                             max_active=8, min_subset=C4_SUBSET_MIN, precision=args.precision,
                             precond_rank=args.stream_precond)
    finally:
        st.close()
    out.update({"workload": C4.name, "n": C4.n, "m": C4.m, "build_s": round(build_s, 2),
                "note": f"first {args.c4_stream} requests of the 512-request c4 stream"})
    return out


METRIC = ("REML fits/hr, p50/p99 latency: mixed-precision batched serving form "
          "(plain FP32 single-fit form alongside), 1 GB300, |dh2|<1e-3")


def fit_counts(wl):
    """Operator applications and right-hand-side columns per fit of the
    workload, as counted by a GPU serving run of this benchmark
    (``--write-counts``), committed under profiles/."""
    path = os.path.join(ROOT, "profiles", f"fit_counts_{wl.name}.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        c = json.load(f)
    return float(c["operator_apps_per_fit"]), float(c["rhs_columns_per_fit"]), path


def run_reference(args, wl):
    ws, rank, _ = _dist()
    if rank != 0:
        return None
    # The reference (jax + numba) is not installable here; its CPU path is
    # restated by the oracle and run on all host cores.  Each step: one whole
    # fit of the small CPU-runnable configuration (measured end to end), and
    # the workload's fit extrapolated from one operator application on a
    # 1,024-SNP call block at n samples, scaled by the per-fit operator counts
    # of this benchmark's GPU serving run.
    from coherit_gb300.configs import C1

    whole = wl.name == C1.name
    counts = None if whole else fit_counts(wl)
    if counts is None and not whole:
        return {"impl": "reference",
                "unavailable": f"no per-fit operator counts for {wl.name} under profiles/"}
    for _ in range(args.warmup):
        cpu_operator_sample(wl.n, 256, 4, wl.seed, reps=1)
    times, c1 = [], []
    for _ in range(args.steps):
        c1.append(cpu_c1_fit()[0])
        if whole:
            times.append(c1[-1])
            continue
        t_fit, cores, sample = cpu_fit_estimate(wl, counts[0], counts[1])
        times.append(t_fit)
    t_fit = statistics.median(times)
    value = 3600.0 / t_fit
    if whole:
        cores = _cores()
        sample = ("whole fit of the CPU port (FP32 kv_impl_streamed on 4,096-SNP packed calls, "
                  "affine SLQ cache, block PCG, AI-REML), measured end to end")
    else:
        sample += f" (counts: {os.path.relpath(counts[2], ROOT)})"
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 5),
        "unit": "fits/hr",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_fit * 1e3, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 (reference arithmetic, CPU)",
        "data": "synthetic (MAF~U(0.05,0.5) HWE genotypes)",
        "config": {"workload": wl.name, "n": wl.n, "m": wl.m, "slq_probes": wl.slq_samples,
                   "lanczos_steps": wl.slq_m, "covariates": wl.n_covar, "pcg_tol": wl.pcg_tol,
                   "parallelism": "CPU, one fit at a time"},
        "cpu_baseline": {"value": round(value, 5), "unit": "fits/hr", "cores": cores,
                         "kind": "port", "extrapolated": not whole, "sample": sample,
                         "c1_whole_fit_s": round(statistics.median(c1), 2)},
        "e2e": {"value": round(value, 5), "unit": "fits/hr", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_c3(args, wl):
    """The 8-component workload (``--config c3``): n x m block-LD genotypes
    generated on the device, 8 components = 4 MAF bins x 2 LD-score halves
    (LD scores from the first 4,096 samples), per-component h2 ~ Dirichlet(1)
    x 0.4 from n_causal / 8 causal SNPs each, 10 covariates, 128 SLQ probes,
    projected-core preconditioner; fits one at a time through the model API
    (the serving loop takes single-component genotypes).  Reports the cold
    and warm fit times, the operator roofline at the SLQ width (128) and at
    the PCG width, and the plain FP32 fit extrapolated from its per-application
    times and the mixed fit's operator counts (a full FP32 fit at this size
    takes tens of minutes)."""
    import torch

    from coherit_gb300 import synth
    from coherit_gb300.geno_stream import GenoBlockStreamer, LDBlockSource

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    hbm_peak, tensor_peak, peak_src = _peaks(sustained=True)
    t0 = time.perf_counter()
    groups, tables = synth.ld_partition_device(wl.seed, wl.m, block=wl.ld_block, device=dev)
    st = GenoBlockStreamer(LDBlockSource(wl.n, wl.m, seed=wl.seed, block=wl.ld_block),
                           component_variant_indices=groups, device=dev,
                           precision=args.precision)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    G = len(groups)
    h2s = synth.dirichlet_h2(wl.seed, G, total=wl.h2_dirichlet_total)
    rng = np.random.default_rng(wl.seed + 1)
    starts = np.concatenate([[0], np.cumsum([g.size for g in groups])])
    fits = 2
    ys, Xs = [], []
    for r in range(fits):
        B = np.zeros((st.m, G), np.float32)
        for g in range(G):
            pos = rng.choice(groups[g].size, size=min(wl.n_causal // G, groups[g].size),
                             replace=False)
            B[starts[g] + pos, g] = rng.normal(size=pos.size)
        gv = st.zxb(torch.as_tensor(B, device=dev)).double()
        gv = gv * torch.sqrt(torch.as_tensor(h2s, device=dev) / gv.var(dim=0, unbiased=False))
        gen = torch.Generator(device=dev).manual_seed(wl.seed + 7 * r)
        noise = torch.randn(st.n, generator=gen, device=dev, dtype=torch.float64)
        ys.append((gv.sum(dim=1) + noise * math.sqrt(1.0 - h2s.sum())).float())
        X = torch.randn((st.n, wl.n_covar + 1), generator=gen, device=dev)
        X[:, 0] = 1.0
        Xs.append(X)
    # The whole probe block per Lanczos sweep: 128 probes x 31 vectors of
    # n floats (plus the reverse pass) fit a 24 GiB SLQ workspace.
    slq_ws = int(min(24 * 1024 ** 3, torch.cuda.mem_get_info(dev)[0] // 4))
    fitter = make_fitter(st, wl, args.precision, slq_workspace_bytes=slq_ws)
    sampler = ClockSampler(0)
    sampler.start()
    times, res = [], []
    for r in range(fits):
        a0, k0 = st.op_stats["apps"], st.op_stats["cols"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res.append(fitter.fit_infinitesimal(ys[r], Xs[r]))
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t0, st.op_stats["apps"] - a0,
                      st.op_stats["cols"] - k0))
    clocks = sampler.stop()
    warm_s, apps, cols = times[-1]
    roof_slq = operator_roofline(st, wl.slq_samples, hbm_peak, tensor_peak, reps=3,
                                 precision=args.precision)
    k_pcg = wl.n_covar + 2
    roof_pcg = operator_roofline(st, k_pcg, hbm_peak, tensor_peak, reps=3,
                                 precision=args.precision)
    fp32_slq = operator_roofline(st, wl.slq_samples, hbm_peak, tensor_peak, reps=1,
                                 precision="fp32")
    fp32_pcg = operator_roofline(st, k_pcg, hbm_peak, tensor_peak, reps=2, precision="fp32")
    # FP32 fit time from the mixed fit's counts: wide (SLQ) and narrow
    # applications priced at their own FP32 times.
    mixed_ratio = fp32_pcg["ms_per_application"] / roof_pcg["ms_per_application"]
    fp32_fit_s = warm_s * max(mixed_ratio, fp32_slq["ms_per_application"] /
                              roof_slq["ms_per_application"]) if apps else None
    st.close()
    return {
        "metric": "REML fits/hr, 8-component block-LD workload (single fits, model API)",
        "value": round(3600.0 / warm_s, 3), "unit": "fits/hr", "higher_is_better": True,
        "config": {"workload": wl.name, "n": wl.n, "m": wl.m, "components": G,
                   "slq_probes": wl.slq_samples, "lanczos_steps": wl.slq_m,
                   "precision": args.precision, "precond_rank": wl.precond_rank,
                   "slq_workspace_bytes": slq_ws},
        "build_s": round(build_s, 2), "cold_fit_s": round(times[0][0], 2),
        "warm_fit_s": round(warm_s, 2), "operator_apps_per_fit": apps,
        "rhs_columns_per_fit": cols,
        "h2_true_total": round(float(h2s.sum()), 4),
        "h2": [round(r.heritability, 4) for r in res],
        "var_components": [[round(float(v), 5) for v in r.var_components] for r in res],
        "component_sizes": [int(g.size) for g in groups],
        "roofline_slq_width": roof_slq, "roofline_pcg_width": roof_pcg,
        "plain_fp32": {"ms_per_application_slq_width": fp32_slq["ms_per_application"],
                       "ms_per_application_pcg_width": fp32_pcg["ms_per_application"],
                       "fit_s_extrapolated": None if fp32_fit_s is None else round(fp32_fit_s, 1),
                       "note": "extrapolated: the mixed fit's time scaled by the FP32/mixed "
                               "per-application ratio (the larger of the SLQ and PCG widths)"},
        "clocks": clocks, "peak_source": peak_src,
    }


def run_operator_only(args, wl):
    """Operator micro-benchmark: W + K applications of K V at width
    ``--operator`` on the workload's genotypes (or --n/--m), CUDA-event timed
    on the launching stream.  Used for kernel profiles."""
    import dataclasses

    import torch

    from coherit_gb300 import _lib

    if args.n or args.m:
        wl = dataclasses.replace(wl, name=f"n{args.n or wl.n}_m{args.m or wl.m}",
                                 n=args.n or wl.n, m=args.m or wl.m, components=None)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    hbm_peak, tensor_peak, peak_src = _peaks()
    st = build_problem(wl, dev)
    k = args.operator
    V = torch.randn(st.n, k, device=dev)
    for _ in range(args.warmup):
        st.kv(V, precision=args.precision)
    torch.cuda.synchronize()
    l0 = _lib.load().coherit_launch_count()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(0)
    sampler.start()
    e0.record(stream)
    for _ in range(args.steps):
        st.kv(V, precision=args.precision)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    launches = _lib.load().coherit_launch_count() - l0
    alg_bytes = st.n * ((st.m + 3) // 4) + 8 * st.n * k + 8 * st.m
    st.check()
    st.close()
    return {"metric": "genotype operator application time", "value": round(ms, 4), "unit": "ms",
            "higher_is_better": False, "steps": args.steps, "warmup": args.warmup,
            "precision": args.precision,
            "config": {"workload": wl.name, "n": wl.n, "m": wl.m, "k": k},
            "hbm_gbs": round(alg_bytes / (ms * 1e-3) / 1e9, 1),
            "tensor_tflops": round(4.0 * wl.n * wl.m * k / (ms * 1e-3) / 1e12, 1),
            "gpu_launches": int(launches), "clocks": clocks, "peak_source": peak_src}


def smile_problem(n, m, block, dev):
    """The c5 operator: MAF/HWE genotypes (seed 5), m/block blocks with
    W_b ~ Wishart(block, I)/block in FP32 (seeded), kernel-trace
    normalisation.  Returns (streamer, operator, build seconds)."""
    import torch

    from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
    from coherit_gb300.smile_block_w import SmileBlockWeightedOperator

    if m % block:
        raise ValueError("m must be a multiple of the 500-SNP block size")
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=5), device=dev, precision="bf16x3")
    rng = np.random.default_rng(5)
    Ws = []
    for _ in range(m // block):
        A = rng.standard_normal((block, block), dtype=np.float32)
        Ws.append((A @ A.T / np.float32(block)).astype(np.float32))
    t0 = time.perf_counter()
    op = SmileBlockWeightedOperator(st, Ws, normalization="kernel_trace", diag_mode="mean")
    torch.cuda.synchronize()
    return st, op, time.perf_counter() - t0


def run_lambda_path(args, wl):
    """c5's weighted-LASSO V^-1 work along a 20-point lambda path
    (``--lambda-path``): the SMILE operator at n=100,000 x m=300,000 (600
    blocks of 500 SNPs, or --n/--m), H = theta_g K + theta_e I with the
    kernel trace-normalised (theta_g = theta_e = 0.5), phenotype from 200
    causal SNPs with Laplace(0, 0.1) effects at h2 0.5 plus an intercept.
    A screening solve H^-1 [y, 1] gives the projected score |Z^T P y|
    (lasso_cd.py:791-822); along the path the next 64 markers by score enter
    the candidate set at each point and their standardised columns are
    solved as one 64-column batched PCG (run_sparse_reml_pipeline.py:
    1202-1297, :2300-2380), BF16x3 genotype tiles, tol 1e-5.  Device time
    of each point's solve with CUDA events on the launching stream; column
    extraction is reported apart."""
    import torch

    from coherit_gb300 import _lib
    from coherit_gb300.hinv import compute_projected_hinv_vector, solve_hinv_columns_batched

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n, m, block = args.n or 100000, args.m or 300000, 500
    points, width, tol, maxiter = 20, 64, 1e-5, 1000
    st, op, build_s = smile_problem(n, m, block, dev)
    rng = np.random.default_rng(55)
    causal = rng.choice(m, size=200, replace=False)
    beta = np.zeros((m, 1), dtype=np.float32)
    beta[causal, 0] = rng.laplace(0.0, 0.1, size=200)
    g = st.zxb(torch.as_tensor(beta, device=dev))[:, 0].double()
    g = (g - g.mean()) / g.std() * np.sqrt(0.5)
    e = torch.as_tensor(rng.standard_normal(n) * np.sqrt(0.5), device=dev)
    y = (g + e).float()
    ones = torch.ones(n, device=dev)
    tg, te = 0.5, 0.5

    def hv(V):
        return tg * op.kv(V) + te * V

    l0 = _lib.load().coherit_launch_count()
    t0 = time.perf_counter()
    sol, sdiag = solve_hinv_columns_batched(hv=hv, precond=None,
                                            rhs=torch.stack([y, ones], dim=1).contiguous(),
                                            warm_start=None, tol=tol, maxiter=maxiter,
                                            batch_size=width, stage="screening")
    u = compute_projected_hinv_vector(covar=np.ones((n, 1)),
                                      Hinv_covar=sol[:, 1:].double().cpu().numpy(),
                                      Hinv_target=sol[:, 0].double().cpu().numpy(), ridge=1e-6)
    score = st.xtv(torch.as_tensor(u, dtype=torch.float32, device=dev)).abs().cpu().numpy()
    order = np.argsort(-score, kind="stable")
    torch.cuda.synchronize()
    screen_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    per_point, iters, extract_s = [], [], 0.0
    for i in range(points):
        markers = np.sort(order[i * width:(i + 1) * width])
        t1 = time.perf_counter()
        Z = st.standardized_columns(markers).contiguous()
        torch.cuda.synchronize()
        extract_s += time.perf_counter() - t1
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, d = solve_hinv_columns_batched(hv=hv, precond=None, rhs=Z, warm_start=None, tol=tol,
                                          maxiter=maxiter, batch_size=width,
                                          stage=f"lambda point {i}")
        e1.record(stream)
        torch.cuda.synchronize()
        per_point.append(round(e0.elapsed_time(e1), 2))
        iters.append(int(d["total_batch_iterations"]))
    launches = _lib.load().coherit_launch_count() - l0
    st.check()
    st.close()
    total_ms = float(sum(per_point))
    return {"metric": "c5 lambda-path V^-1 batched solves (64 RHS per point, 20 points)",
            "value": round(total_ms / 1e3, 3), "unit": "s", "higher_is_better": False,
            "config": {"workload": f"c5_n{n}_m{m}_blocks{m // block}x{block}",
                       "rhs_per_point": width, "points": points, "pcg_tol": tol,
                       "precision": "bf16x3", "theta": [tg, te]},
            "ms_per_point": per_point, "pcg_iterations_per_point": iters,
            "mean_ms_per_point": round(total_ms / points, 1),
            "screening_s": round(screen_s, 3), "screening_iterations":
                int(sdiag["total_batch_iterations"]),
            "column_extraction_s": round(extract_s, 3), "build_s": round(build_s, 2),
            "gpu_launches": int(launches), "data": "synthetic (seeded)"}


def run_smile_only(args, wl):
    """SMILE block-weighted operator at the c5 shape (``--smile K``): n=100,000
    x m=300,000 (or --n/--m), blocks of 500 SNPs with W_b ~ Wishart(500, I)/500
    in FP32 (seeded), kernel-trace normalisation; K V at width K timed with
    CUDA events on the launching stream.  Algorithmic work: the two genome
    contractions (4nmk flops, n*ceil(m/4) genotype bytes) plus the W_b
    products (2*m*500*k flops, 4*500*m bytes of W)."""
    import torch

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n, m, block, k = args.n or 100000, args.m or 300000, 500, args.smile
    hbm_peak, tensor_peak, peak_src = _peaks()
    st, op, build_s = smile_problem(n, m, block, dev)
    V = torch.randn(n, k, device=dev)
    for _ in range(max(3, args.warmup)):
        op.kv(V)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        op.kv(V)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    flops = 4.0 * n * m * k + 2.0 * m * block * k
    nbytes = n * ((m + 3) // 4) + 4 * block * m + 8 * n * k + 8 * m
    tfs = flops / (ms * 1e-3) / 1e12
    st.close()
    return {"metric": "SMILE block-weighted operator application time", "value": round(ms, 4),
            "unit": "ms", "higher_is_better": False, "steps": args.steps,
            "config": {"workload": f"c5_n{n}_m{m}_blocks{m // block}x{block}", "k": k},
            "build_s": round(build_s, 2),
            "roofline": {"bound": "tensor", "achieved": round(tfs, 1), "peak": tensor_peak,
                         "unit": "TFLOP/s", "frac": round(tfs / tensor_peak, 4), "traffic": None,
                         "algorithmic_flops": flops, "algorithmic_bytes": nbytes,
                         "hbm_gbs": round(nbytes / (ms * 1e-3) / 1e9, 1)},
            "peak_source": peak_src}


def run_stream_only(args, wl):
    """Only the Poisson request stream (``--stream-only``) on the workload's
    matrix, e.g. a prefix of the c4 serving stream (``--config c4``: n=200,000
    x m=600,000, subsets log-uniform in [1e4, 2e5])."""
    import torch

    from coherit_gb300.configs import C4_SUBSET_MIN

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    t0 = time.perf_counter()
    st = build_problem(wl, dev)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    sampler = ClockSampler(0)
    sampler.start()
    out = serving_stream(st, wl, args.stream, args.stream_rate, seed=wl.seed + 99,
                         max_active=args.requests,
                         min_subset=C4_SUBSET_MIN if wl.name.startswith("c4") else None,
                         precision=args.precision, precond_rank=args.stream_precond)
    clocks = sampler.stop()
    st.close()
    out.update({"metric": "REML fits/hr over a Poisson request stream", "config": wl.name,
                "n": wl.n, "m": wl.m, "build_s": round(build_s, 2), "clocks": clocks})
    return out


def run_mma_rate(args, wl):
    """Tensor-core issue-rate table (``--mma-rate``): cycles per tcgen05.mma
    (M = 128, A in tensor memory) by operand kind, width N and issuing threads
    per SM, with the aggregate rate of all SMs (CUDA events) as TFLOP/s.  The
    operator's narrow launches are bound by this rate, not by HBM."""
    import ctypes as C

    import torch

    from coherit_gb300 import _lib

    torch.cuda.set_device(0)
    lib = _lib.load()
    iters = 1 << 14
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    _, tensor_peak, peak_src = _peaks()
    rows = []
    for kind, kname, kk in ((0, "bf16", 16), (1, "e4m3", 32)):
        for issuers in (1, 2):
            for n in (16, 32, 48, 64, 80, 96, 128, 160, 192, 224, 256):
                if issuers == 2 and n > 224:
                    continue
                cyc, ms = C.c_double(), C.c_double()
                _lib.check(lib.coherit_mma_rate(kind, n, issuers, iters, C.byref(cyc),
                                                C.byref(ms), _lib.stream_ptr()), "mma rate")
                flops = 2.0 * 128 * n * kk * iters * issuers * sms
                rows.append({"kind": kname, "N": n, "issuers": issuers,
                             "cycles_per_mma": round(cyc.value, 1),
                             "tflops": round(flops / (ms.value * 1e-3) / 1e12, 1)})
    return {"metric": "tcgen05.mma issue rate", "unit": "cycles per instruction",
            "iters": iters, "sms": sms, "peak_tflops": tensor_peak, "peak_source": peak_src,
            "rows": rows}


def run_sparse_only(args, wl):
    """Rare-variant operator micro-benchmark (``--sparse K``) at the
    workload's n x m (or --n/--m), as reported in the ``sparse12`` object of
    the full run.  Used for kernel profiles."""
    import torch

    torch.cuda.set_device(0)
    n, m = args.n or wl.n, args.m or wl.m
    hbm_peak, _, peak_src = _peaks()
    out = sparse12_operator(n, m, args.sparse, hbm_peak, float("nan"), seed=wl.seed + 7,
                            reps=max(1, args.steps))
    out.pop("dense_kv_ms_same_shape")
    out["peak_source"] = peak_src
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c3s")
    ap.add_argument("--precision", default="auto",
                    help="operator precision: auto (fp8x5 up to 48 columns, bf16x3 above), "
                         "bf16x3, fp8x5, fp16x2")
    ap.add_argument("--requests", type=int, default=8,
                    help="concurrent fit requests per step (the serving batch)")
    ap.add_argument("--stream", type=int, default=24,
                    help="requests in the Poisson-arrival subset stream (0 = skip)")
    ap.add_argument("--stream-rate", type=float, default=2.0,
                    help="stream arrivals per second (Poisson)")
    ap.add_argument("--stream-precond", type=int, default=0,
                    help="projected-core preconditioner rank of the streamed fits (0 = none)")
    ap.add_argument("--c4-stream", type=int, default=16,
                    help="requests of the c4 serving stream (200k x 600k) run after the "
                         "headline workload (0 = skip)")
    ap.add_argument("--c4-rate", type=float, default=0.5,
                    help="c4 stream arrivals per second (Poisson)")
    ap.add_argument("--batch-window", type=float, default=0.01,
                    help="seconds the batcher waits for the other active fits")
    ap.add_argument("--single-fits", type=int, default=3,
                    help="fits timed one at a time for the single-fit comparison")
    ap.add_argument("--no-single", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the fixed launch policy (no tuning of the launch widths)")
    ap.add_argument("--sparse12", action="store_true",
                    help="also time the rare-variant (sparse12) operator at the workload's size")
    ap.add_argument("--write-counts", default="",
                    help="write the per-fit operator counts of the timed fits to this JSON file")
    ap.add_argument("--operator", type=int, default=0, metavar="K",
                    help="time bare operator applications of width K instead of fits")
    ap.add_argument("--smile", type=int, default=0, metavar="K",
                    help="time the SMILE block-weighted operator (c5 shape) at width K")
    ap.add_argument("--stream-only", action="store_true",
                    help="run only the Poisson request stream on the workload's matrix")
    ap.add_argument("--sparse", type=int, default=0, metavar="K",
                    help="time the rare-variant operator at width K instead of fits")
    ap.add_argument("--lambda-path", action="store_true",
                    help="time c5's 20-point lambda path of 64-column V^-1 solves")
    ap.add_argument("--mma-rate", action="store_true",
                    help="print the tensor-core instruction issue-rate table")
    ap.add_argument("--n", type=int, default=0, help="with --operator/--sparse: samples")
    ap.add_argument("--m", type=int, default=0, help="with --operator/--sparse: SNPs")
    args = ap.parse_args()
    from coherit_gb300.configs import WORKLOADS

    wl = WORKLOADS[args.config]
    if args.mma_rate:
        out = run_mma_rate(args, wl)
    elif args.lambda_path:
        out = run_lambda_path(args, wl)
    elif args.operator > 0:
        out = run_operator_only(args, wl)
    elif args.sparse > 0:
        out = run_sparse_only(args, wl)
    elif args.stream_only:
        out = run_stream_only(args, wl)
    elif args.smile > 0:
        out = run_smile_only(args, wl)
    elif args.impl == "reference":
        out = run_reference(args, wl)
    elif wl.partition == "maf_ld":
        out = run_c3(args, wl)
    else:
        out = run_ours(args, wl)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
