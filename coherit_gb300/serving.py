"""Continuous-batching REML serving over one resident genotype matrix.

Requests (a phenotype, optional covariates and an optional sample subset)
are admitted while active slots and the HBM budget allow.  Every admitted
request runs the ordinary ``fit_reml`` (strict AI-REML, affine SLQ) in its
own worker thread; its genotype-operator applications do not launch kernels
themselves but are handed to a batcher, which concatenates the pending
right-hand sides of all active requests column-wise and applies the operator
to all of them in one ``coherit_geno_kv_batched`` launch (each request with
its own statistics slot -- mean, inverse sd and m_eff over its sample subset
-- its own scale theta_g/m_eff and residual weight theta_e).  A request that
arrives while others are in flight is admitted as soon as a slot frees up,
and its operator work joins the running fits' launches.

A request over a sample subset S is solved in the compressed index space of
S (vectors of length |S|); the batcher scatters them into the n-row block
and gathers the rows of S back, which is exactly K_S = Z_S Z_S^T / m_eff(S)
with Z_S standardised over S -- the matrix a streamer built on the subset
(``GenoBlockStreamer(..., sample_mask=S)``, geno_stream.py:1230-1247) applies.

All device work goes to the device's default stream, so the batched launches
and the fits' own tensor arithmetic are ordered without extra events.  Calls
into the genotype library on the shared handle are serialised by one lock.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import threading
import time
from collections import deque
from concurrent.futures import Future
from typing import Optional

import numpy as np
import torch

from . import _lib
from .geno_stream import GenoBlockStreamer
from .precond import ProjectedCorePrecondConf, build_lowrank_basis
from .reml import REMLProbeCache, fit_reml, prime_probe_cache

# Widest right-hand-side block one batched launch takes per precision: the
# split terms of all columns sit side by side in one MMA (N <= 256).
_MAX_BATCH_COLS = {"bf16x3": 80, "bf16x2": 128, "bf16x1": 256, "fp16x2": 128, "fp8x5": 48,
                   "auto": 80}


@dataclasses.dataclass
class ServeResult:
    request_id: int
    var_components: np.ndarray
    heritability: float
    loglik: float
    n_samples: int
    arrival: float
    start: float
    finish: float
    history: list

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


@dataclasses.dataclass
class _Request:
    rid: int
    y: np.ndarray
    covar: Optional[np.ndarray]
    mask: Optional[np.ndarray]
    arrival: float
    future: Future
    fit_kwargs: dict
    n_sub: int
    bytes_estimate: int
    slot: int = 0
    idx: Optional[torch.Tensor] = None
    eff: float = 0.0
    atom: float = 0.0


@dataclasses.dataclass
class _Target:
    """Where an operator application goes: stats slot, subset rows, row count."""
    slot: int
    idx: Optional[torch.Tensor]
    n_sub: int


class _Op:
    __slots__ = ("req", "V", "scale", "theta_e", "done", "out", "error", "next_col", "cols_done")

    def __init__(self, req, V, scale, theta_e):
        self.req = req
        self.V = V
        self.scale = scale
        self.theta_e = theta_e
        self.done = threading.Event()
        self.out = None
        self.error = None
        self.next_col = 0   # first column not yet placed in a launch
        self.cols_done = 0  # columns whose results are back


class _Batcher:
    """Collects operator applications of concurrent fits into batched launches.

    A launch goes out when every active fit has an application pending;
    otherwise, while the previous launch still runs on the device, the
    batcher keeps gathering (a launch now would only queue behind it), and
    from the moment the device has finished it waits at most ``window_s``
    for the fits that launch served to submit again.  Launches are filled to ``max_cols`` columns: an application whose block
    does not fit the rest of a launch is split by columns, its first columns
    riding in this launch and the others in the next (the operator acts on
    columns independently), so every launch but the last of a round streams
    the genotypes for a full-width block.
    """

    def __init__(self, streamer: GenoBlockStreamer, precision: str, window_s: float,
                 max_cols: int, lib_lock: threading.Lock, launch_ms: dict | None = None):
        self.st = streamer
        self.prec = _lib.PRECISIONS[precision]
        self.window_s = float(window_s)
        self.max_cols = int(max_cols)
        # Measured time of one launch per width (multiples of 16): the
        # pending columns are then cut into the launches of least total time.
        self.launch_ms = {int(w): float(t) for w, t in (launch_ms or {}).items()
                          if int(w) % 16 == 0 and 0 < int(w) <= self.max_cols}
        self.lib_lock = lib_lock
        self.cv = threading.Condition()
        self.pending: list[_Op] = []
        self.n_active = 0
        self.stop = False
        self.launches = 0
        self.columns = 0
        self.requests_per_launch: list[int] = []
        self.last_launch: torch.cuda.Event | None = None  # completion of the latest launch
        # (start, end) events of the latest launches (launch number
        # _events_base + index): device time of the operator.
        self.launch_events: list[tuple] = []
        self._events_base = 0
        self.launch_widths: list[int] = []  # columns of the latest launches (bounded)
        self._busy_cap_s = 0.25  # longest wait for stragglers while the device is busy
        self.thread = threading.Thread(target=self._loop, name="coherit-batcher", daemon=True)
        self.thread.start()

    def set_active(self, delta: int) -> None:
        with self.cv:
            self.n_active += delta
            self.cv.notify_all()

    def apply(self, req, V: torch.Tensor, scale: float, theta_e) -> torch.Tensor:
        vec = V.ndim == 1
        V2 = (V[:, None] if vec else V).to(torch.float32).contiguous()
        if V2.shape[0] != req.n_sub:
            raise ValueError(f"V has {V2.shape[0]} rows, the request has {req.n_sub} samples")
        op = _Op(req, V2, float(scale), None if theta_e is None else float(theta_e))
        op.out = torch.empty_like(V2)
        if V2.shape[1] == 0:
            return op.out[:, 0] if vec else op.out
        with self.cv:
            if self.stop:
                raise RuntimeError("REMLServer is closed.")
            self.pending.append(op)
            self.cv.notify_all()
        op.done.wait()
        if op.error is not None:
            raise op.error
        return op.out[:, 0] if vec else op.out

    def device_ms(self, first: int = 0) -> float:
        """Device time of launch number `first` onwards, as far as their events
        are kept (synchronises with the last one)."""
        evs = self.launch_events[max(0, first - self._events_base):]
        if not evs:
            return 0.0
        evs[-1][1].synchronize()
        return float(sum(a.elapsed_time(b) for a, b in evs))

    def close(self) -> None:
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        self.thread.join(timeout=30)

    def _take(self) -> list[tuple]:
        """Pieces (op, first column, last column + 1) of the next launch."""
        with self.cv:
            while not self.pending and not self.stop:
                self.cv.wait()
            if not self.pending:
                return []
            start = time.perf_counter()
            idle_since = None
            while len(self.pending) < self.n_active and not self.stop:
                now = time.perf_counter()
                # While the previous launch still runs on the device a launch
                # now would only queue behind it: keep gathering.  The fits it
                # serves submit again shortly after it completes, so the
                # window for them opens when the device finishes.
                if self.last_launch is not None and not self.last_launch.query():
                    idle_since = None
                    if now - start >= self._busy_cap_s:
                        break
                    self.cv.wait(timeout=0.0005)
                    continue
                if idle_since is None:
                    idle_since = now
                left = self.window_s - (now - idle_since)
                if left <= 0:
                    break
                self.cv.wait(timeout=min(left, 0.0005))
            width = self._first_width(sum(op.V.shape[1] - op.next_col for op in self.pending))
            pieces, cols = [], 0
            while self.pending and cols < width:
                op = self.pending[0]
                lo = op.next_col
                hi = min(op.V.shape[1], lo + width - cols)
                pieces.append((op, lo, hi))
                cols += hi - lo
                op.next_col = hi
                if hi == op.V.shape[1]:
                    self.pending.pop(0)
            return pieces

    def _first_width(self, total: int) -> int:
        """Width of the next launch: max_cols, or with measured launch times
        the first launch of the cheapest cut of `total` pending columns into
        launches of the measured widths (the last may be padded)."""
        if not self.launch_ms or total <= 0:
            return self.max_cols
        widths = sorted(self.launch_ms)
        units = -(-total // 16)
        best = [0.0] + [float("inf")] * units
        first = [0] * (units + 1)
        for u in range(1, units + 1):
            for w in widths:
                rest = max(0, u - w // 16)
                t = self.launch_ms[w] + best[rest]
                if t < best[u]:
                    best[u], first[u] = t, w
        return max(16, min(first[units] or self.max_cols, self.max_cols))

    def _loop(self) -> None:
        while True:
            pieces = self._take()
            if not pieces:
                return
            try:
                self._launch(pieces)
            except BaseException as err:  # handed to every fit in the launch
                with self.cv:
                    for op, _, _ in pieces:
                        op.error = err
                        if op in self.pending:
                            self.pending.remove(op)
                for op, _, _ in pieces:
                    op.done.set()
                continue
            for op, lo, hi in pieces:
                op.cols_done += hi - lo
                if op.cols_done == op.V.shape[1]:
                    op.done.set()

    def _launch(self, pieces: list[tuple]) -> None:
        st = self.st
        widths = [hi - lo for _, lo, hi in pieces]
        K = int(sum(widths))
        col_start = np.zeros(len(pieces) + 1, dtype=np.int32)
        col_start[1:] = np.cumsum(widths)
        Vf = torch.zeros((st.n, K), dtype=torch.float32, device=st.dev)
        for (op, lo, hi), c0 in zip(pieces, col_start[:-1]):
            if op.req.idx is None:
                Vf[:, c0:c0 + hi - lo] = op.V[:, lo:hi]
            else:
                Vf[op.req.idx, c0:c0 + hi - lo] = op.V[:, lo:hi]
        slots = np.asarray([op.req.slot for op, _, _ in pieces], dtype=np.int32)
        scale = np.asarray([op.scale for op, _, _ in pieces], dtype=np.float32)
        te = np.asarray([0.0 if op.theta_e is None else op.theta_e for op, _, _ in pieces],
                        dtype=np.float32)
        out = torch.empty_like(Vf)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        with self.lib_lock:
            _lib.check(_lib.load().coherit_geno_kv_batched(
                st.handle, len(pieces), col_start.ctypes.data, slots.ctypes.data, self.prec,
                Vf.data_ptr(), K, K, scale.ctypes.data, te.ctypes.data, out.data_ptr(), K,
                _lib.stream_ptr()), "batched kv")
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        self.last_launch = ev
        self.launch_events.append((ev0, ev))
        self.launch_widths.append(K)
        if len(self.launch_events) > 8192:  # bounded: keep the latest half
            drop = len(self.launch_events) // 2
            del self.launch_events[:drop]
            del self.launch_widths[:drop]
            self._events_base += drop
        st.op_stats["apps"] += 1
        st.op_stats["cols"] += K
        self.launches += 1
        self.columns += K
        self.requests_per_launch.append(len({id(op) for op, _, _ in pieces}))
        for (op, lo, hi), c0 in zip(pieces, col_start[:-1]):
            blk = out[:, c0:c0 + hi - lo]
            op.out[:, lo:hi] = blk if op.req.idx is None else blk[op.req.idx]


def _init_device_linalg(dev) -> None:
    """Run each device linear-algebra routine a fit uses once on this thread.

    PyTorch loads its CUDA linear-algebra backend lazily on first use, and
    that first use is not safe to race from several threads ("lazy wrapper
    should be called at most once"); the worker threads start only after
    this has run."""
    for dt in (torch.float32, torch.float64):
        A = torch.eye(4, dtype=dt, device=dev) * 2.0
        L, _ = torch.linalg.cholesky_ex(A)
        torch.linalg.cholesky(A)
        torch.cholesky_solve(torch.ones((4, 1), dtype=dt, device=dev), L)
        torch.linalg.eigh(A)
        torch.linalg.qr(A)
    torch.cuda.synchronize(dev)


class REMLServer:
    """Serve single-GRM REML fits of many phenotypes over one resident matrix.

    ``max_active`` bounds the fits in flight; ``hbm_budget_bytes`` bounds the
    device memory their solver state may take (estimated per request from its
    sample count and right-hand-side width; default half the free memory).
    ``fit_kwargs`` go to ``fit_reml`` (defaults: 30 trace probes, 30 SLQ
    probes x 30 Lanczos steps, PCG tol 1e-5, 20 AI iterations).

    ``launch_ms`` ({width: ms}, e.g. from ``GenoBlockStreamer.autotune``)
    lets the batcher cut the pending right-hand sides into the launches of
    least measured total time instead of filling ``max_batch_cols`` first.
    Off by default: with 8 single-GRM fits at n = 100k, m = 1M it measured
    10.8k against 11.3k fits/hr (76 launches of 38 columns per step against
    61 of 48: rounds that are not complete yet get cut narrow).

    ``precond_rank`` > 0 gives every fit's PCG solves a projected-core
    preconditioner of that rank (reml_model.py:863-960, single GRM): a
    Nystrom basis U of the request's own kernel (K over its sample subset)
    from two operator applications of width rank + 8, which join the other
    fits' launches, and the core diag(eigenvalues) - atom I.  Full-cohort
    requests share one.  It changes how fast PCG converges, not the
    solutions it converges to; the SLQ log-determinant is not preconditioned
    (the affine SLQ form takes none).
    """

    def __init__(self, streamer: GenoBlockStreamer, *, max_active: int = 8,
                 hbm_budget_bytes: float | None = None, precision: str = "bf16x3",
                 batch_window_s: float = 0.01, max_batch_cols: int | None = None,
                 fit_kwargs: dict | None = None, precond_rank: int = 0,
                 launch_ms: dict | None = None):
        if streamer.n_components != 1:
            raise ValueError("REMLServer serves single-GRM fits (one genotype component).")
        if precision not in _MAX_BATCH_COLS:
            raise ValueError(f"precision must be one of {sorted(_MAX_BATCH_COLS)}")
        if max_active < 1:
            raise ValueError("max_active must be >= 1")
        self.st = streamer
        self.max_active = int(max_active)
        if hbm_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(streamer.dev)
            hbm_budget_bytes = 0.5 * free
        self.budget = float(hbm_budget_bytes)
        self.precision = precision
        self._lib_lock = threading.Lock()
        # Statistics slots 1..max_active serve subset requests; creating the
        # highest one first sizes the handle's slot table once.
        self._free_slots = deque(range(1, self.max_active + 1))
        with self._lib_lock:
            _lib.check(_lib.load().coherit_geno_compute_stats(
                streamer.handle, self.max_active, None, None, None, None, _lib.stream_ptr()),
                "reserve stats slots")
        _init_device_linalg(streamer.dev)
        cols = _MAX_BATCH_COLS[precision] if max_batch_cols is None else int(max_batch_cols)
        self.batcher = _Batcher(streamer, precision, batch_window_s, cols, self._lib_lock,
                                launch_ms=launch_ms)
        self.fit_kwargs = dict(n_rand_vec=30, maxiter=500, minq_iter=20, slq_samples=30,
                               slq_m=30, pcg_tol=1e-5, verbose=False)
        if fit_kwargs:
            self.fit_kwargs.update(fit_kwargs)
        # Full-cohort requests share one operator (slot 0) and so one set of
        # phenotype-independent probe work (the affine SLQ Lanczos data),
        # built by the first such request and reused by the rest, as the
        # single-fit path reuses it across phenotypes (reml.py:62-73).
        self._full = _Target(slot=0, idx=None, n_sub=streamer.n)
        inv_full = 1.0 / streamer._eff_m_host if streamer._eff_m_host > 0 else 1.0
        self._full_K = lambda V: self.batcher.apply(self._full, V, inv_full, None)
        self._full_cache = REMLProbeCache()
        self._full_cache_key = None
        self._full_cache_lock = threading.Lock()
        self.precond_rank = max(0, int(precond_rank))
        self._full_precond = None
        self._full_precond_lock = threading.Lock()
        self._cv = threading.Condition()
        self._waiting: deque[_Request] = deque()
        self._active = 0
        self._bytes_active = 0.0
        self._next_id = 0
        self._closed = False
        self.results: list[ServeResult] = []
        self._admitter = threading.Thread(target=self._admit_loop, name="coherit-admit",
                                          daemon=True)
        self._admitter.start()

    # -------------------------------------------------------------- requests
    def submit(self, y, covar=None, sample_mask=None, **fit_kwargs) -> Future:
        """Queue one fit; returns a Future resolving to a ServeResult.

        ``y`` and ``covar`` have one row per selected sample (all samples of
        the resident matrix when ``sample_mask`` is None)."""
        if self._closed:
            raise RuntimeError("REMLServer is closed.")
        mask = None
        n_sub = self.st.n
        if sample_mask is not None:
            mask = np.asarray(sample_mask, dtype=bool).reshape(-1)
            if mask.size != self.st.n:
                raise ValueError(f"sample_mask has {mask.size} entries, the matrix has "
                                 f"{self.st.n} samples")
            n_sub = int(mask.sum())
            if n_sub == 0:
                raise ValueError("sample_mask selects no samples")
        # Host arrays are copied to the device by the fit; device tensors stay.
        if isinstance(y, torch.Tensor):
            y = y.detach().to(self.st.dev, torch.float32).reshape(-1)
        else:
            y = np.asarray(y, dtype=np.float32).reshape(-1)
        if y.shape[0] != n_sub:
            raise ValueError(f"phenotype has {y.shape[0]} entries, the sample set has {n_sub}")
        if covar is not None:
            if isinstance(covar, torch.Tensor):
                covar = covar.detach().to(self.st.dev, torch.float32)
            else:
                covar = np.asarray(covar, dtype=np.float32)
            if covar.ndim == 1:
                covar = covar[:, None]
            if covar.shape[0] != n_sub:
                raise ValueError("covariates must have one row per selected sample")
        kw = dict(self.fit_kwargs)
        kw.update(fit_kwargs)
        p = 0 if covar is None else covar.shape[1]
        width = p + 1 + int(kw.get("n_rand_vec", 30)) + int(kw.get("slq_samples", 30))
        # Solver state: a few n x width FP32 blocks (solutions, residuals,
        # directions, operator outputs) plus the Lanczos basis of the probes.
        est = 4 * n_sub * (8 * width + int(kw.get("slq_m", 30)) * int(kw.get("slq_samples", 30)))
        fut: Future = Future()
        with self._cv:
            rid = self._next_id
            self._next_id += 1
            self._waiting.append(_Request(rid=rid, y=y, covar=covar, mask=mask,
                                          arrival=time.perf_counter(), future=fut,
                                          fit_kwargs=kw, n_sub=n_sub, bytes_estimate=est))
            self._cv.notify_all()
        return fut

    def map(self, requests) -> list[ServeResult]:
        """Submit (y, covar, sample_mask) tuples and wait for all results."""
        futs = [self.submit(*r) for r in requests]
        return [f.result() for f in futs]

    def stats(self) -> dict:
        lat = np.asarray([r.latency for r in self.results], dtype=np.float64)
        out = {"completed": int(lat.size), "launches": self.batcher.launches,
               "columns": self.batcher.columns,
               "mean_requests_per_launch": float(np.mean(self.batcher.requests_per_launch))
               if self.batcher.requests_per_launch else 0.0}
        if lat.size:
            out.update(p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)))
        return out

    def close(self) -> None:
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        self._admitter.join(timeout=30)
        self.batcher.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------- admission
    def _can_admit(self, req: _Request) -> bool:
        if self._active >= self.max_active:
            return False
        if req.mask is not None and not self._free_slots:
            return False
        return self._active == 0 or self._bytes_active + req.bytes_estimate <= self.budget

    def _admit_loop(self) -> None:
        while True:
            with self._cv:
                while not self._closed and not (self._waiting and
                                                self._can_admit(self._waiting[0])):
                    self._cv.wait()
                if self._closed:
                    for req in self._waiting:
                        req.future.set_exception(RuntimeError("REMLServer is closed."))
                    self._waiting.clear()
                    return
                req = self._waiting.popleft()
                self._active += 1
                self._bytes_active += req.bytes_estimate
                if req.mask is not None:
                    req.slot = self._free_slots.popleft()
            self.batcher.set_active(+1)
            threading.Thread(target=self._run, args=(req,), name=f"coherit-fit-{req.rid}",
                             daemon=True).start()

    def _release(self, req: _Request) -> None:
        self.batcher.set_active(-1)
        with self._cv:
            self._active -= 1
            self._bytes_active -= req.bytes_estimate
            if req.slot > 0:
                self._free_slots.append(req.slot)
            self._cv.notify_all()

    # ------------------------------------------------------------------- fit
    def _prepare(self, req: _Request) -> None:
        st = self.st
        if req.mask is None:
            req.eff = st._eff_m_host
            req.atom = st._mean_diag_atom_host
            return
        lib = _lib.load()
        mask_u8 = np.ascontiguousarray(req.mask, dtype=np.uint8)
        ce = np.zeros(st.n_components)
        ca = np.zeros(st.n_components)
        et, at = C.c_double(), C.c_double()
        with self._lib_lock:
            _lib.check(lib.coherit_geno_compute_stats(
                st.handle, req.slot, mask_u8.ctypes.data, None, None, None, _lib.stream_ptr()),
                "request stats")
            _lib.check(lib.coherit_geno_stats_summary(st.handle, req.slot, ce.ctypes.data,
                                                      ca.ctypes.data, C.byref(et), C.byref(at)),
                       "request stats summary")
        req.eff, req.atom = float(et.value), float(at.value)
        req.idx = torch.as_tensor(np.flatnonzero(req.mask), dtype=torch.long, device=st.dev)

    def _projected_core(self, K, req: _Request):
        """Projected-core preconditioner of one request's kernel K (single
        GRM, reml_model.py:863-960 with uniform reference weight 1): Nystrom
        basis U, eigenvalues e of U^T K U, core diag(e) - atom I, identity
        diagonal atom."""
        dev = self.st.dev
        rank = int(min(self.precond_rank, req.n_sub))
        seed = int(req.fit_kwargs.get("seed", 0))
        U, evals = build_lowrank_basis(K, req.n_sub, rank, key=seed + 4321, device=dev)
        r = int(U.shape[1])
        eye = torch.eye(r, dtype=U.dtype, device=dev)
        core = torch.diag(evals.to(U.dtype))[None] - float(req.atom) * eye[None]
        return ProjectedCorePrecondConf(
            U=U, core_atoms=core, total_rank=r, n_grm=1, diag_mode="scalar_identity",
            diag_atoms=torch.tensor([req.atom], dtype=torch.float32, device=dev),
            residual_diag_atoms=torch.ones(1, dtype=torch.float32, device=dev), identity=eye)

    def _precond_for(self, req: _Request, K):
        if self.precond_rank <= 0:
            return None
        if req.mask is not None:
            return self._projected_core(K, req)
        with self._full_precond_lock:
            if self._full_precond is None:
                self._full_precond = self._projected_core(self._full_K, req)
            return self._full_precond

    def _shared_cache_key(self, req: _Request):
        """(seed, slq_samples, slq_m) when the request may use the shared
        full-cohort probe cache, else None (subset requests, caller-supplied
        probes or cache, other optimizers)."""
        kw = req.fit_kwargs
        if req.mask is not None or kw.get("slq_probes") is not None or "probe_cache" in kw:
            return None
        if kw.get("optimizer", "strict") != "strict" or kw.get("slq_mode", "raw") != "raw":
            return None
        return (int(kw.get("seed", 0)), int(kw.get("slq_samples", 30)), int(kw.get("slq_m", 30)))

    def _run(self, req: _Request) -> None:
        start = time.perf_counter()
        try:
            torch.cuda.set_device(self.st.dev)
            self._prepare(req)
            b = self.batcher
            inv_eff = 1.0 / req.eff if req.eff > 0 else 1.0

            def whv(theta_g, theta_e, V):
                tg = float(np.asarray(theta_g, dtype=np.float64).reshape(-1)[0])
                return b.apply(req, V, tg * inv_eff, float(theta_e))

            kw = dict(req.fit_kwargs)
            cache_key = self._shared_cache_key(req)
            shared = False
            if cache_key is not None:
                # The first full-cohort request builds the cache (its
                # applications batch with the other fits); later ones wait
                # here and reuse it.  Another probe setting keeps its own.
                with self._full_cache_lock:
                    if self._full_cache_key is None:
                        prime_probe_cache(self._full_cache, self._full_K, req.n_sub,
                                          seed=cache_key[0], slq_samples=cache_key[1],
                                          slq_m=cache_key[2], device=self.st.dev)
                        self._full_cache_key = cache_key
                    shared = self._full_cache_key == cache_key
            if shared:
                K_mvs = [self._full_K]
                kw["probe_cache"] = self._full_cache
            else:
                K_mvs = [lambda V: b.apply(req, V, inv_eff, None)]
            diag = torch.tensor(req.atom, dtype=torch.float32, device=self.st.dev)
            if "precond_conf" not in kw:
                kw["precond_conf"] = self._precond_for(req, K_mvs[0])
            param, hist, d = fit_reml(req.y, K_mvs, [diag], req.covar, weighted_hv=whv,
                                      device=self.st.dev, return_diagnostics=True, **kw)
            gen = float(np.dot(param[:1], np.asarray(d.get("genetic_trace_atoms", [1.0]))))
            res = float(np.dot(param[1:], np.asarray(d.get("residual_trace_atoms", [1.0]))))
            out = ServeResult(request_id=req.rid, var_components=np.asarray(param),
                              heritability=gen / max(gen + res, 1e-12),
                              loglik=float(d["loglik"]), n_samples=req.n_sub,
                              arrival=req.arrival, start=start, finish=time.perf_counter(),
                              history=hist)
            with self._cv:
                self.results.append(out)
            req.future.set_result(out)
        except BaseException as err:
            req.future.set_exception(err)
        finally:
            self._release(req)


__all__ = ["REMLServer", "ServeResult"]
