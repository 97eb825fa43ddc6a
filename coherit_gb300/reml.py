"""REML fitting by AI-REML / Fisher scoring on the GPU operator.

Mirrors GPU_REML's reml.py (fit_reml :1254-2092, _eval_once :685-971):

* the phenotype is standardised once (reml.py:151-163);
* every objective evaluation solves H [X | y (| probes)] = rhs by block PCG
  with the projected-core preconditioner, projects out the fixed effects
  through the FP64 Cholesky of X^T H^-1 X (reml.py:780-801), and evaluates
  ll = -(y'Py + log|H| + log|X^T H^-1 X|) / (2n);
* log|H| is the affine single-GRM SLQ (one Lanczos run on K reused for every
  theta, reml.py:367-486) or the multi-component fixed-probe SLQ with its
  exact gradient (reml.py:489-540);
* the score is (y'P K_i P y - d logdet_i) / (2n) and the average-information
  matrix 1/2 (G P y)^T P (G P y) / n (reml.py:938-953);
* the bound-constrained Fisher step is solved through NNLS with a KKT
  active-set polish in FP64 (reml.py:979-1131), followed by a strict
  backtracking line search (reml.py:1695-1880).

Device work: operator applications, PCG, Lanczos and the n x k products.
FP64 on the device: X^T H^-1 X and its Cholesky, the projected products, the
tridiagonal eigensolves and the log-likelihood sums.  The (G+E)-sized NNLS
runs on the host in FP64 as in the reference.
"""
from __future__ import annotations

import logging
import math
import time
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np
import scipy.linalg as sla
import torch
from scipy.optimize import nnls

from .pcg import pcg_solve
from .precond import (
    ProjectedCorePrecondConf,
    ProjectedCoreRuntime,
    build_projected_core_runtime,
    make_precond,
    make_projected_core_precond_from_runtime,
    projected_core_apply_invsqrt,
    projected_core_logdet,
    scalar_diag_from_precond_conf,
)
from .slq import logdet_value_and_grad as _slq_value_and_grad
from .slq import rademacher

logger = logging.getLogger(__name__)

FI_SYSTEM_RIDGE = 1e-4
F32_EPS = float(np.finfo(np.float32).eps)


@dataclass(frozen=True)
class AffineSLQCache:
    """Lanczos coefficients for theta_g K + theta_e I log-determinants (reml.py:52-59)."""

    alphas_k: torch.Tensor  # (m, S) FP64
    betas_k: torch.Tensor   # (m-1, S) FP64
    z_norm_sq: float
    nsamples_f: float


@dataclass
class REMLProbeCache:
    """Response/theta-independent work reused across fits (reml.py:62-73)."""

    signature: tuple | None = None
    kvrand_stack: torch.Tensor | None = None
    affine_slq: AffineSLQCache | None = None


@dataclass
class REMLContext:
    n: int
    G: int
    E: int
    K_mvs: tuple
    weighted_hv: Optional[Callable]
    stacked_kv: Optional[Callable]
    diag_stack: Optional[torch.Tensor]
    residual_diag_stack: Optional[torch.Tensor]
    xmat: Optional[torch.Tensor]
    y: torch.Tensor
    rhs_const: torch.Tensor
    y_col: int
    rand_stop: int
    n_XyZ_cols: int
    R_rand: int
    kvrand_stack: Optional[torch.Tensor]
    precond_conf: Optional[ProjectedCorePrecondConf]
    diag_atoms: Optional[np.ndarray] = None
    residual_diag_atoms: Optional[np.ndarray] = None
    affine_slq_cache: Optional[AffineSLQCache] = None
    slq_reference_runtime: Optional[ProjectedCoreRuntime] = None
    slq_workspace_bytes: int = 256 * 1024 ** 2
    slq_probes: Optional[torch.Tensor] = None


@dataclass
class FisherSolveStats:
    free_dim: int = 0
    frozen_genetic: int = 0
    ai_pcg_iters: int = 0
    ai_elapsed_sec: float = 0.0
    ws_resolve_count: int = 0
    ws_fixed_total: int = 0
    ws_released_total: int = 0
    ws_trace: str = ""

    def to_dict(self) -> dict:
        return dict(self.__dict__)


@dataclass
class AverageInfoMatrix:
    mat: np.ndarray
    ridge: float = FI_SYSTEM_RIDGE
    stats: Optional[FisherSolveStats] = None


# ------------------------------------------------------------------ helpers

def standardize_response(y):
    """(y - mean) / (std + 1e-6) in FP32 (reml.py:151-163)."""
    y = torch.as_tensor(y, dtype=torch.float32).reshape(-1)
    if y.numel() == 0:
        raise ValueError("Phenotype must contain at least one sample.")
    if not bool(torch.all(torch.isfinite(y))):
        raise ValueError("Phenotype contains non-finite values.")
    y_mean = torch.mean(y)
    y_std = torch.std(y, unbiased=False)
    if not bool(torch.isfinite(y_std)) or float(y_std) <= 0.0:
        raise ValueError("Phenotype must have positive finite variance.")
    y_scale = y_std + 1e-6
    return (y - y_mean) / y_scale, y_mean, y_scale


def _validate_fixed_effect_design(xmat: torch.Tensor, *, relative_tol: float = 1e-7) -> None:
    """Reject zero or collinear fixed-effect columns (reml.py:166-184)."""
    X = xmat.double()
    gram = (X.T @ X).cpu().numpy()
    norms_sq = np.diag(gram)
    if not np.all(np.isfinite(norms_sq)) or np.any(norms_sq <= 0.0):
        raise ValueError("covar contains a zero or non-finite fixed-effect column.")
    norms = np.sqrt(norms_sq)
    corr = gram / (norms[:, None] * norms[None, :])
    ev = np.linalg.eigvalsh(0.5 * (corr + corr.T))
    if ev[0] <= float(relative_tol) * max(float(ev[-1]), 1.0):
        raise ValueError(
            "covar is rank-deficient or numerically collinear; "
            "remove redundant fixed-effect columns."
        )


def _mean_diag_atoms(diag_list, *, n_samples=None) -> np.ndarray:
    """tr(K_i)/n from scalar or per-sample diagonals (reml.py:187-212)."""
    atoms = []
    for i, d in enumerate(diag_list):
        arr = np.asarray(d.detach().cpu() if isinstance(d, torch.Tensor) else d, dtype=np.float32)
        if arr.ndim not in (0, 1):
            raise ValueError(f"diag_list[{i}] must be scalar or one-dimensional.")
        if arr.ndim == 1 and n_samples is not None and arr.size != n_samples:
            raise ValueError(
                f"diag_list[{i}] length mismatch: expected {int(n_samples)}, got {int(arr.size)}."
            )
        if not (np.all(np.isfinite(arr)) and np.all(arr >= 0)):
            raise ValueError("diag_list entries must contain finite nonnegative values.")
        atoms.append(float(arr) if arr.ndim == 0 else float(np.mean(arr, dtype=np.float32)))
    return np.asarray(atoms, dtype=np.float64)


def _scalar_diag_from_diag_list(diag_list):
    atoms = []
    for d in diag_list:
        arr = np.asarray(d.detach().cpu() if isinstance(d, torch.Tensor) else d, dtype=np.float32)
        if arr.size == 0:
            atoms.append(0.0)
            continue
        flat = arr.reshape(-1)
        if not np.all(flat == flat[0]):
            return None
        atoms.append(float(flat[0]))
    return np.asarray(atoms, dtype=np.float64)


def _stable_cho_factor_spd(A: torch.Tensor, *, base_jitter=1e-6, max_tries=8) -> torch.Tensor:
    """FP64 Cholesky with geometric jitter escalation (reml.py:240-277)."""
    A = 0.5 * (A + A.T)
    p = A.shape[0]
    if p == 0:
        raise ValueError("stable_cho_factor_spd requires a non-empty square matrix.")
    scale = float(torch.mean(torch.abs(torch.diagonal(A))))
    if not math.isfinite(scale) or scale <= 0.0:
        scale = 1.0
    eye = torch.eye(p, dtype=A.dtype, device=A.device)
    for k in range(-1, max_tries):
        jit = 0.0 if k < 0 else base_jitter * scale * (10.0 ** k)
        L, info = torch.linalg.cholesky_ex(A + jit * eye)
        d = torch.diagonal(L)
        if int(info) == 0 and bool(torch.all(torch.isfinite(d)) and torch.all(d > 0)):
            return L
    raise FloatingPointError("Failed to stabilize XtHinvX Cholesky with jitter escalation.")


def _tridiag(alphas: torch.Tensor, betas: torch.Tensor) -> torch.Tensor:
    m, S = alphas.shape
    T = torch.zeros((S, m, m), dtype=torch.float64, device=alphas.device)
    idx = torch.arange(m, device=alphas.device)
    T[:, idx, idx] = alphas.T.double()
    if m > 1:
        off = torch.arange(m - 1, device=alphas.device)
        T[:, off + 1, off] = betas.T.double()
        T[:, off, off + 1] = betas.T.double()
    return T


# ------------------------------------------------------------ affine SLQ

def _lanczos_step(v, w_raw, prev, beta_prev):
    """Fused Lanczos recurrence with local orthogonalisation (reml.py:285-304)."""
    w = w_raw - prev * beta_prev[None, :]
    alpha = torch.sum(v.double() * w.double(), dim=0)
    w = w - v * alpha.float()[None, :]
    norm = torch.sqrt(torch.sum(w.double() * w.double(), dim=0))
    safe = torch.where(norm > 0, norm, torch.ones_like(norm))
    return (w / safe.float()[None, :]), alpha, norm


def _build_affine_slq_cache(K_fn, n_dim, key, *, nsamples, m, probes=None, device=None):
    """Run Lanczos once on K for the affine pencil (reml.py:367-412)."""
    dev = device if device is not None else torch.device("cuda")
    z = rademacher(n_dim, nsamples, key, dev) if probes is None else probes.to(dev, torch.float32)
    v = (z / math.sqrt(float(n_dim))).contiguous()
    alphas, betas = [], []
    prev = torch.zeros_like(v)
    beta_prev = torch.zeros(nsamples, dtype=torch.float32, device=dev)
    for i in range(m):
        w_raw = torch.as_tensor(K_fn(v), dtype=torch.float32, device=dev)
        v_next, alpha, norm = _lanczos_step(v, w_raw, prev, beta_prev)
        alphas.append(alpha)
        if i < m - 1:
            betas.append(norm)
        prev, beta_prev, v = v, norm.float(), v_next.contiguous()
    A = torch.stack(alphas)
    B = torch.stack(betas) if betas else torch.zeros((0, nsamples), dtype=torch.float64, device=dev)
    return AffineSLQCache(alphas_k=A, betas_k=B, z_norm_sq=float(n_dim), nsamples_f=float(nsamples))


def _affine_slq_logdet(cache: AffineSLQCache, theta_g, theta_e, *, return_derivatives=False):
    """logdet(theta_g T_K + theta_e I) and its derivatives (reml.py:415-486)."""
    T = _tridiag(cache.alphas_k, cache.betas_k)
    m = cache.alphas_k.shape[0]
    ev, vec = torch.linalg.eigh(T)
    w = vec[:, 0, :] ** 2
    raw = float(theta_g) * ev + float(theta_e)
    floor = max(F32_EPS * m, 1e-6)
    h = torch.clamp(raw, min=floor)
    factor = cache.z_norm_sq / cache.nsamples_f
    logdet = factor * torch.sum(w * torch.log(h))
    if not return_derivatives:
        return logdet
    active = (raw > floor).double()
    d_scale = factor * torch.sum(w * active * ev / h)
    d_shift = factor * torch.sum(w * active / h)
    return logdet, torch.stack([d_scale, d_shift])


# -------------------------------------------------------- operators / stacks

def _as_col(v):
    return v[:, None] if v.ndim == 1 else v


def _hv_apply(K_mvs, theta_g, theta_e, V, residual_diag_stack=None):
    """H V = sum theta_g[i] K_i V + sum theta_e[j] R_j V (reml.py:547-565)."""
    if residual_diag_stack is None:
        acc = float(theta_e[0]) * V
    else:
        rd = torch.tensordot(torch.as_tensor(theta_e, dtype=torch.float32, device=V.device),
                             residual_diag_stack, dims=1)
        acc = rd[:, None] * _as_col(V)
        if V.ndim == 1:
            acc = acc[:, 0]
    for i, mv in enumerate(K_mvs):
        if float(theta_g[i]) != 0.0:
            acc = acc + float(theta_g[i]) * mv(V)
    return acc


def _apply_genetic_stack(ctx: REMLContext, V, component_idx=None):
    if component_idx is None and ctx.stacked_kv is not None:
        return ctx.stacked_kv(V)
    idx = range(ctx.G) if component_idx is None else component_idx
    return torch.stack([_as_col(ctx.K_mvs[int(i)](V)) for i in idx], dim=0)


def _apply_residual_stack(ctx: REMLContext, V):
    Vm = _as_col(V)
    if ctx.residual_diag_stack is None:
        return Vm[None, :, :]
    return ctx.residual_diag_stack[:, :, None] * Vm[None, :, :]


def _residual_diag_from_components(ctx: REMLContext, theta_e):
    te = np.asarray(theta_e, dtype=np.float64).reshape(-1)
    if ctx.residual_diag_stack is None:
        return float(te[0])
    return torch.tensordot(torch.as_tensor(te, dtype=torch.float32, device=ctx.y.device),
                           ctx.residual_diag_stack, dims=1)


def _compute_traces_from_pcg(sol_all, ctx: REMLContext):
    """Hutchinson tr(H^-1 R_j), tr(H^-1 K_i) from PCG probe columns (reml.py:608-649)."""
    a, b = ctx.y_col + 1, ctx.rand_stop
    HinvV = sol_all[:, a:b].double()
    Vr = ctx.rhs_const[:, a:b].double()
    R = float(ctx.R_rand)
    if ctx.residual_diag_stack is None:
        trR = (torch.sum(Vr * HinvV) / R).reshape(1)
    else:
        trR = torch.einsum("nr,en,nr->e", Vr, ctx.residual_diag_stack.double(), HinvV) / R
    trK = torch.einsum("nr,inr->i", HinvV, ctx.kvrand_stack.double()) / R
    return trR, trK


def _compute_score_traces(ctx: REMLContext, PZrand, Vrand):
    """SMILE score traces tr(P K_i), tr(P R_j) from cached K_i Vrand (reml.py:652-682)."""
    R = float(ctx.R_rand)
    tg = torch.einsum("nr,inr->i", PZrand.double(), ctx.kvrand_stack.double()) / R
    if ctx.residual_diag_stack is None:
        tr = (torch.sum(Vrand.double() * PZrand.double()) / R).reshape(1)
    else:
        tr = torch.einsum("nr,en,nr->e", Vrand.double(), ctx.residual_diag_stack.double(),
                          PZrand.double()) / R
    return torch.cat([tg, tr])


def _multi_slq_logdet_and_score(ctx: REMLContext, Hv_fn, pvec, key, *, nsamples, m,
                                use_reference, accept_logdet=None):
    """Fixed-probe SLQ of (optionally whitened) H and its exact gradient (reml.py:489-540)."""
    reference = ctx.slq_reference_runtime if use_reference else None
    pv = np.asarray(pvec, dtype=np.float64)

    def whiten(v):
        return projected_core_apply_invsqrt(reference, v) if reference is not None else v

    def Bv(v):
        return whiten(Hv_fn(whiten(v)))

    def pullback(left, right):
        left, right = whiten(left), whiten(right)
        result = torch.zeros_like(left)
        scores = []
        stack = _apply_genetic_stack(ctx, left)
        for k in range(ctx.G):
            product = stack[k]
            result = result + float(pv[k]) * product
            scores.append(torch.sum(right.double() * product.double()))
        for e in range(ctx.E):
            product = left if ctx.residual_diag_stack is None else ctx.residual_diag_stack[e, :, None] * left
            result = result + float(pv[ctx.G + e]) * product
            scores.append(torch.sum(right.double() * product.double()))
        return whiten(result), torch.stack(scores)

    ref_ld = projected_core_logdet(reference, ctx.n).double() if reference is not None else 0.0
    value, gradient = _slq_value_and_grad(
        Bv, pullback, ctx.n, key, nsamples=nsamples, m=m,
        workspace_bytes=ctx.slq_workspace_bytes, dtype=torch.float32,
        accept_value=(None if accept_logdet is None else
                      (lambda v: accept_logdet(v + ref_ld))),
        device=ctx.y.device, probes=ctx.slq_probes,
    )
    return value + ref_ld, gradient


# ---------------------------------------------------------------- eval_once

def _eval_once(ctx: REMLContext, pvec, warm_all, warm_ai=None, *, key_slq, minq_tol, maxiter,
               precond_eps, slq_samples, slq_m, slq_mode="raw", warm_ready=False,
               warm_ai_ready=False, taylor_logdet=None, compute_traces=True, min_loglik=None):
    """One REML objective evaluation (reml.py:685-971)."""
    pvec = np.asarray(pvec, dtype=np.float64)
    theta_g = pvec[: ctx.G]
    theta_e = pvec[ctx.G:]
    dev = ctx.y.device

    def Hv(V):
        if ctx.weighted_hv is not None:
            te = theta_e[0] if ctx.E == 1 else theta_e
            return ctx.weighted_hv(theta_g, te, V)
        return _hv_apply(ctx.K_mvs, theta_g, theta_e, V, ctx.residual_diag_stack)

    tg_t = torch.as_tensor(theta_g, dtype=torch.float32, device=dev)
    te_t = torch.as_tensor(theta_e, dtype=torch.float32, device=dev)
    diag_H = scalar_diag_from_precond_conf(ctx.precond_conf, tg_t, te_t)
    if diag_H is None:
        if ctx.diag_atoms is not None:
            diag_H = _residual_diag_from_components(ctx, theta_e) + float(np.dot(theta_g, ctx.diag_atoms))
        else:
            if ctx.diag_stack is None:
                raise ValueError(
                    "diag_stack is required when the preconditioner does not provide a scalar diagonal."
                )
            diag_H = _residual_diag_from_components(ctx, theta_e) + torch.tensordot(
                tg_t, ctx.diag_stack, dims=1)
    use_residual_slq = bool(slq_mode == "projected_core_residual" and taylor_logdet is None
                            and ctx.affine_slq_cache is None
                            and ctx.slq_reference_runtime is not None)
    runtime = build_projected_core_runtime(ctx.precond_conf, tg_t, diag_H, eps=precond_eps,
                                           need_invsqrt=False)
    if runtime is not None:
        M_cur = make_projected_core_precond_from_runtime(runtime)
    else:
        M_cur = make_precond(ctx.precond_conf, tg_t, diag_H, eps=precond_eps)

    rhs_all = ctx.rhs_const
    if warm_ready:
        X0_all = warm_all
    elif M_cur is not None:
        X0_all = M_cur(rhs_all)
    else:
        X0_all = torch.zeros_like(rhs_all)
    sol_all, main_rel, k_pcg = pcg_solve(Hv, rhs_all, M=M_cur, tol=minq_tol, maxiter=maxiter,
                                         X0=X0_all)
    main_rel_h = float(main_rel)
    if not math.isfinite(main_rel_h) or main_rel_h > minq_tol * 1.05:
        raise FloatingPointError(
            "Main REML PCG did not converge: "
            f"relative residual={main_rel_h:.3e}, tolerance={minq_tol:.3e}, "
            f"iterations={int(k_pcg)}/{int(maxiter)}."
        )
    warm_all_next = sol_all

    HinvXyZ = sol_all[:, : ctx.n_XyZ_cols]
    chol = None
    if ctx.xmat is not None and ctx.xmat.shape[1] > 0:
        x_cols = ctx.xmat.shape[1]
        Xd = ctx.xmat.double()
        HinvX = HinvXyZ[:, :x_cols].double()
        chol = _stable_cho_factor_spd(Xd.T @ HinvX)

        def proj(mat):
            mid = torch.cholesky_solve(Xd.T @ mat.double(), chol)
            return (mat.double() - HinvX @ mid)
    else:
        HinvX = None

        def proj(mat):
            return mat.double()

    PYstar = proj(HinvXyZ[:, ctx.y_col: ctx.rand_stop])
    Py = PYstar[:, :1]
    yPy = torch.dot(ctx.y.double(), PYstar[:, 0])
    logdet_x = (2.0 * torch.sum(torch.log(torch.clamp(torch.diagonal(chol), min=1e-30)))
                if chol is not None else torch.zeros((), dtype=torch.float64, device=dev))
    n_f = float(ctx.n)

    def loglik(logdet_value):
        return -0.5 * (yPy + logdet_value + logdet_x) / n_f

    trace_sel = None
    if taylor_logdet is not None:
        logdet = taylor_logdet
    elif ctx.affine_slq_cache is not None:
        logdet, trace_sel = _affine_slq_logdet(ctx.affine_slq_cache, theta_g[0], theta_e[0],
                                               return_derivatives=True)
    else:
        logdet, trace_sel = _multi_slq_logdet_and_score(
            ctx, Hv, pvec, key_slq, nsamples=slq_samples, m=slq_m,
            use_reference=use_residual_slq,
            accept_logdet=(None if min_loglik is None else
                           (lambda v: bool(float(loglik(v)) >= min_loglik))),
        )
    ll = loglik(logdet)
    ll_h = float(ll)
    if not math.isfinite(ll_h):
        raise FloatingPointError("Non-finite REML objective.")
    if min_loglik is not None and not ll_h >= min_loglik:
        return (ll_h, None, None, int(k_pcg), warm_all_next, None, None, None, logdet)

    Pyf = Py.float().contiguous()
    GPy_gen = _apply_genetic_stack(ctx, Pyf)
    GPy_res = _apply_residual_stack(ctx, Pyf)
    GPy_stack = torch.cat([GPy_gen, GPy_res], dim=0)
    q_sel = torch.einsum("n,in->i", Py[:, 0], GPy_stack[:, :, 0].double())
    if taylor_logdet is not None:
        trace_sel = _compute_score_traces(ctx, PYstar[:, 1:],
                                          ctx.rhs_const[:, ctx.y_col + 1: ctx.rand_stop])
    elif ctx.affine_slq_cache is not None:
        if HinvX is not None:
            K_HinvX = _apply_genetic_stack(ctx, HinvX.float().contiguous())[0].double()
            rhs = [HinvX.T @ K_HinvX, HinvX.T @ HinvX]
            correction = torch.stack([torch.trace(torch.cholesky_solve(r, chol)) for r in rhs])
        else:
            correction = torch.zeros(2, dtype=torch.float64, device=dev)
        trace_sel = trace_sel - correction
    else:
        if HinvX is not None:
            Kst = _apply_genetic_stack(ctx, HinvX.float().contiguous())
            rhs = [HinvX.T @ Kst[g].double() for g in range(ctx.G)]
            for e in range(ctx.E):
                prod = HinvX if ctx.residual_diag_stack is None else \
                    ctx.residual_diag_stack[e, :, None].double() * HinvX
                rhs.append(HinvX.T @ prod)
            correction = torch.stack([torch.trace(torch.cholesky_solve(r, chol)) for r in rhs])
            trace_sel = trace_sel - correction

    stats = FisherSolveStats(free_dim=ctx.G + ctx.E)
    GPy_cols = GPy_stack[:, :, 0].T.contiguous()
    if warm_ai_ready and warm_ai is not None and warm_ai.shape[1] == ctx.G + ctx.E:
        X0_ai = warm_ai
    elif M_cur is not None:
        X0_ai = M_cur(GPy_cols)
    else:
        X0_ai = torch.zeros_like(GPy_cols)
    t0 = time.perf_counter()
    HinvGPy, ai_rel, k_ai = pcg_solve(Hv, GPy_cols, M=M_cur, tol=minq_tol, maxiter=maxiter,
                                      X0=X0_ai)
    ai_rel_h = float(ai_rel)
    if not math.isfinite(ai_rel_h) or ai_rel_h > minq_tol * 1.05:
        raise FloatingPointError(
            "Average-information PCG did not converge: "
            f"relative residual={ai_rel_h:.3e}, tolerance={minq_tol:.3e}, "
            f"iterations={int(k_ai)}/{int(maxiter)}."
        )
    stats.ai_pcg_iters = int(k_ai)
    stats.ai_elapsed_sec = time.perf_counter() - t0
    PGPy = proj(HinvGPy)
    if compute_traces and ctx.R_rand > 0:
        tr_R, tr_K = _compute_traces_from_pcg(sol_all, ctx)
    else:
        tr_R = tr_K = None
    AI = 0.5 * (GPy_cols.double().T @ PGPy) / n_f
    AI = 0.5 * (AI + AI.T)
    grad = 0.5 * (q_sel - trace_sel.double()) / n_f
    AI_h = AI.cpu().numpy()
    grad_h = grad.cpu().numpy()
    if not (np.all(np.isfinite(AI_h)) and np.all(np.isfinite(grad_h))):
        raise FloatingPointError("Non-finite REML objective, score, or AI matrix.")
    FI = AverageInfoMatrix(mat=AI_h, stats=stats)
    return (ll_h, grad_h, FI, int(k_pcg), warm_all_next, HinvGPy, tr_R, tr_K, logdet)


# --------------------------------------------------------- bound-constrained step

def _freeze_mask(theta_g, grad_g, zero_tol):
    return np.logical_and(np.asarray(theta_g) <= zero_tol, np.asarray(grad_g) <= 0.0)


def _solve_average_info_bound_qp(param, grad, FI: AverageInfoMatrix, *, lower_step,
                                 initial_active, trial_alpha, bound_tol):
    """Bound-constrained Fisher QP through NNLS + KKT active-set polish (reml.py:979-1131)."""
    param = np.asarray(param, np.float64)
    grad = np.asarray(grad, np.float64)
    mat = np.asarray(FI.mat, np.float64)
    lower = np.asarray(lower_step, np.float64)
    n_param = param.size
    if mat.shape != (n_param, n_param):
        raise ValueError("Average-information matrix shape does not match the parameter vector.")
    if not (np.all(np.isfinite(grad)) and np.all(np.isfinite(mat)) and np.all(np.isfinite(lower))):
        raise FloatingPointError("Non-finite value in the bound-constrained Fisher system.")
    ridge = float(FI.ridge)
    if not math.isfinite(ridge) or ridge < 0.0:
        raise ValueError("Average-information ridge must be finite and nonnegative.")
    system = 0.5 * (mat + mat.T) + ridge * np.eye(n_param)
    scale = float(np.mean(np.abs(np.diag(system))))
    if not math.isfinite(scale) or scale <= 0.0:
        scale = 1.0
    chol = None
    solved = system
    for attempt in range(9):
        jit = 0.0 if attempt == 0 else 1e-8 * scale * (10.0 ** (attempt - 1))
        cand = system if jit == 0.0 else system + jit * np.eye(n_param)
        try:
            chol = sla.cholesky(cand, lower=True, check_finite=False)
            solved = cand
            break
        except np.linalg.LinAlgError:
            continue
    if chol is None:
        raise FloatingPointError("Failed to stabilize the bound-constrained Fisher system.")
    shifted_rhs = grad - solved @ lower
    target = sla.solve_triangular(chol, shifted_rhs, lower=True, check_finite=False)
    shifted, _ = nnls(chol.T, target, maxiter=max(3 * n_param, 1))
    ptol = max(float(bound_tol), 1e-10)
    active = float(trial_alpha) * shifted <= ptol
    shifted[active] = 0.0
    kkt_scale = max(1.0, float(np.max(np.abs(grad), initial=0.0)))
    kkt_tol = max(1e-7, 1e-6 * kkt_scale)
    for _ in range(max(5 * n_param, 1)):
        free = ~active
        shifted.fill(0.0)
        if np.any(free):
            try:
                fc = sla.cho_factor(solved[np.ix_(free, free)], lower=True, check_finite=False)
                shifted[free] = sla.cho_solve(fc, shifted_rhs[free], check_finite=False)
            except np.linalg.LinAlgError as err:
                raise FloatingPointError("Failed to polish the NNLS Fisher active set.") from err
            nonpos = free & (shifted <= 0.0)
            if np.any(nonpos):
                active[nonpos] = True
                continue
        resid = shifted_rhs - solved @ shifted
        viol = active & (resid > kkt_tol)
        if np.any(viol):
            cands = np.flatnonzero(viol)
            active[int(cands[np.argmax(resid[cands])])] = False
            continue
        break
    else:
        raise FloatingPointError("NNLS Fisher active-set polish did not converge.")
    step = lower + shifted
    kkt = grad - solved @ step
    free = ~active
    free_err = float(np.max(np.abs(kkt[free]), initial=0.0))
    act_err = float(np.max(kkt[active], initial=0.0))
    if free_err > kkt_tol or act_err > kkt_tol:
        raise FloatingPointError(
            "NNLS Fisher solve did not satisfy KKT tolerance: "
            f"free_error={free_err:.3e}, active_error={act_err:.3e}, tolerance={kkt_tol:.3e}."
        )
    unconstrained = sla.cho_solve((chol, True), grad, check_finite=False)
    would_block = unconstrained < lower - ptol
    init = np.asarray(initial_active, dtype=bool).reshape(-1)
    provisional = init | would_block
    return (step, active, int(np.count_nonzero(active & ~init)),
            int(np.count_nonzero(provisional & ~active)))


def _projected_fisher_direction(param, grad, FI: AverageInfoMatrix, *, n_genetic=None,
                                genetic_zero_tol, residual_floor=0.0, trial_alpha=1.0):
    """Projected Fisher-scoring direction (reml.py:1134-1221)."""
    param = np.asarray(param, np.float64)
    grad = np.asarray(grad, np.float64)
    G = param.size - 1 if n_genetic is None else int(n_genetic)
    if G < 0 or G > param.size:
        raise ValueError("n_genetic must be between 0 and len(param).")
    if residual_floor < 0.0:
        raise ValueError("residual_floor must be >= 0.")
    if trial_alpha <= 0.0:
        raise ValueError("trial_alpha must be > 0.")
    active = np.zeros(param.size, dtype=bool)
    active[:G] = _freeze_mask(param[:G], grad[:G], genetic_zero_tol)
    if G < param.size:
        active[G:] = (param[G:] <= residual_floor + genetic_zero_tol) & (grad[G:] <= 0.0)
    lower_param = np.concatenate([np.zeros(G), np.full(param.size - G, residual_floor)])
    lower_step = (lower_param - param) / trial_alpha
    step, final_active, fixed, released = _solve_average_info_bound_qp(
        param, grad, FI, lower_step=lower_step, initial_active=active, trial_alpha=trial_alpha,
        bound_tol=genetic_zero_tol)
    if FI.stats is not None:
        FI.stats.free_dim = int(np.count_nonzero(~final_active))
        FI.stats.frozen_genetic = int(np.count_nonzero(final_active[:G]))
        FI.stats.ws_resolve_count = 1
        FI.stats.ws_fixed_total = fixed
        FI.stats.ws_released_total = released
        FI.stats.ws_trace = (f"solver=nnls free={FI.stats.free_dim} "
                             f"freeze={FI.stats.frozen_genetic} add={fixed} drop={released}")
    return step, final_active[:G]


def _apply_projected_step(param, step_dir, alpha, *, n_genetic=None, genetic_zero_tol,
                          residual_floor):
    """Bounded update theta + alpha d (reml.py:1224-1247)."""
    param = np.asarray(param, np.float64)
    G = param.size - 1 if n_genetic is None else int(n_genetic)
    tg = np.maximum(param[:G] + alpha * step_dir[:G], 0.0)
    tg = np.where(tg <= genetic_zero_tol, 0.0, tg)
    te = np.maximum(param[G:] + alpha * step_dir[G:], residual_floor)
    upd = np.concatenate([tg, te])
    return upd, upd - param


# --------------------------------------------------------------------- fit

def _probe_setup(probe_cache, K_mvs, n, *, seed, Vrand, slq_samples, slq_m, residual_free, E,
                  stacked_kv, slq_probes, dev):
    """Phenotype-independent probe work of a fit: K_i applied to the trace
    probes and the affine SLQ cache, reused when ``probe_cache`` holds them for
    the same operators, sample count, seed and probe shapes (reml.py:62-73)."""
    G = len(K_mvs)
    n_trace = 0 if Vrand is None else int(Vrand.shape[1])
    signature = (K_mvs, n, int(seed), n_trace, int(slq_samples), int(slq_m),
                 bool(residual_free), str(dev))
    hit = probe_cache is not None and probe_cache.signature == signature
    KVrand = probe_cache.kvrand_stack if (hit and Vrand is not None) else None
    if Vrand is not None and KVrand is None:
        KVrand = stacked_kv(Vrand) if stacked_kv is not None else torch.stack(
            [_as_col(mv(Vrand)) for mv in K_mvs])
    affine = probe_cache.affine_slq if hit else None
    if G == 1 and E == 1 and residual_free and affine is None:
        probes = None if slq_probes is None else torch.as_tensor(
            slq_probes, dtype=torch.float32).to(dev)
        key_slq = (int(seed) + 2026) * 3 + 2
        affine = _build_affine_slq_cache(K_mvs[0], n, key_slq, nsamples=slq_samples, m=slq_m,
                                         probes=probes, device=dev)
    if probe_cache is not None:
        probe_cache.signature = signature
        probe_cache.kvrand_stack = KVrand
        probe_cache.affine_slq = affine
    return KVrand, affine


def prime_probe_cache(probe_cache: REMLProbeCache, K_mv: Callable, n: int, *, seed: int = 0,
                      slq_samples: int = 30, slq_m: int = 30, slq_probes=None, device=None):
    """Fill ``probe_cache`` for single-GRM strict fits on ``(K_mv,)``.

    A later ``fit_reml(y, K_mvs, ...)`` with the same tuple object
    ``K_mvs == (K_mv,)``, ``n``, ``seed`` and probe shapes reuses the cached
    affine SLQ data instead of rebuilding it; returns that tuple."""
    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    K_mvs = (K_mv,)
    _probe_setup(probe_cache, K_mvs, int(n), seed=seed, Vrand=None, slq_samples=slq_samples,
                 slq_m=slq_m, residual_free=True, E=1, stacked_kv=None, slq_probes=slq_probes,
                 dev=dev)
    return K_mvs


def fit_reml(
    y,
    K_mvs: Sequence[Callable],
    diag_list: Sequence,
    covar,
    n_rand_vec: int,
    maxiter: int,
    seed: int = 0,
    h2_init: float = 0.5,
    param_init=None,
    minq_iter: int = 50,
    slq_samples: int = 30,
    slq_m: int = 30,
    slq_mode: str = "raw",
    precond_conf: Optional[ProjectedCorePrecondConf] = None,
    slq_precond_conf: Optional[ProjectedCorePrecondConf] = None,
    precond_refresh_fn: Optional[Callable] = None,
    precond_eps: float = 1e-6,
    weighted_hv: Optional[Callable] = None,
    stacked_kv: Optional[Callable] = None,
    residual_diag_list=None,
    residual_floor: float = 1e-2,
    genetic_zero_tol: float = 1e-8,
    max_linesearch_trials: int = 3,
    optimizer: str = "strict",
    scoring_step_tol: float = 1e-4,
    rel_dll_tol: float = 1e-3,
    taylor_threshold: float = 0.01,
    pcg_tol: float = 1e-3,
    response_is_standardized: bool = False,
    unit_variance_components: bool = False,
    verbose: bool = True,
    log_detail: str = "full",
    return_diagnostics: bool = False,
    probe_cache: REMLProbeCache | None = None,
    mean_information=None,
    slq_workspace_bytes: int = 256 * 1024 ** 2,
    device=None,
    slq_probes=None,
    trace_probes=None,
):
    """Single-trait Gaussian REML with AI/Fisher updates (reml.py:1254-2092).

    Returns ``(param, history)`` or ``(param, history, diagnostics)``.
    ``param`` holds (theta_g[0..G), theta_e[0..E)) as a float64 numpy array.
    Probe matrices may be supplied (``slq_probes`` (n, slq_samples),
    ``trace_probes`` (n, n_rand_vec)); otherwise they are drawn from torch
    generators seeded by ``seed`` (the reference derives them from
    jax.random.PRNGKey(seed + 2026)).
    """
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    y = torch.as_tensor(y, dtype=torch.float32).reshape(-1).to(dev)
    n = int(y.shape[0])
    if n <= 0:
        raise ValueError("fit_reml requires at least one phenotype sample.")
    K_mvs = tuple(K_mvs)
    diag_list = tuple(diag_list)
    G = len(K_mvs)
    if G != len(diag_list):
        raise ValueError("Length of K_mvs and diag_list must match.")
    if G == 0:
        raise ValueError("fit_reml requires at least one genetic covariance component.")
    if n_rand_vec <= 0:
        raise ValueError("fit_reml requires n_rand_vec > 0.")
    if maxiter <= 0:
        raise ValueError("fit_reml requires maxiter > 0.")
    if minq_iter < 0:
        raise ValueError("fit_reml requires minq_iter >= 0.")
    if slq_m <= 0:
        raise ValueError("fit_reml requires slq_m > 0.")
    if slq_workspace_bytes < 1:
        raise ValueError("fit_reml requires slq_workspace_bytes > 0.")
    if not 0.0 <= h2_init <= 1.0:
        raise ValueError("h2_init must lie in [0, 1].")
    genetic_atoms = (np.ones(G) if unit_variance_components
                     else _mean_diag_atoms(diag_list, n_samples=n))
    if residual_diag_list is None:
        residual_diag_stack = None
        residual_atoms = np.ones(1)
        E = 1
    else:
        residual_diag_list = tuple(residual_diag_list)
        if not residual_diag_list:
            raise ValueError("residual_diag_list must be non-empty when provided.")
        residual_diag_stack = torch.stack([
            torch.as_tensor(d, dtype=torch.float32).reshape(-1).to(dev) for d in residual_diag_list])
        if residual_diag_stack.shape[1] != n:
            raise ValueError("residual_diag_list entries must have length matching the number of samples.")
        if not bool(torch.all(torch.isfinite(residual_diag_stack))):
            raise ValueError("residual_diag_list contains non-finite values.")
        if bool(torch.any(residual_diag_stack < 0.0)):
            raise ValueError("residual_diag_list entries must be nonnegative.")
        if bool(torch.any(torch.sum(residual_diag_stack, dim=0) <= 0.0)):
            raise ValueError("residual_diag_list must provide positive residual support for every sample.")
        E = int(residual_diag_stack.shape[0])
        residual_atoms = (np.ones(E) if unit_variance_components
                          else residual_diag_stack.double().mean(dim=1).cpu().numpy())
    if slq_samples <= 0:
        raise ValueError("fit_reml requires slq_samples > 0.")
    if slq_mode not in {"raw", "projected_core_residual"}:
        raise ValueError(
            f"Unsupported slq_mode={slq_mode!r}. Expected 'raw' or 'projected_core_residual'.")
    if residual_floor <= 0.0:
        raise ValueError("residual_floor must be > 0.")
    if genetic_zero_tol < 0.0:
        raise ValueError("genetic_zero_tol must be >= 0.")
    if max_linesearch_trials < 1:
        raise ValueError("max_linesearch_trials must be >= 1.")
    if log_detail not in {"compact", "full"}:
        raise ValueError("log_detail must be 'compact' or 'full'.")
    if optimizer not in {"strict", "smile_scoring"}:
        raise ValueError("optimizer must be 'strict' or 'smile_scoring'.")
    if scoring_step_tol < 0.0:
        raise ValueError("scoring_step_tol must be >= 0.")
    if rel_dll_tol < 0.0:
        raise ValueError("rel_dll_tol must be >= 0.")
    if taylor_threshold < 0.0:
        raise ValueError("taylor_threshold must be >= 0.")
    if pcg_tol <= 0.0:
        raise ValueError("pcg_tol must be > 0.")
    if mean_information is not None:
        raise NotImplementedError("sparse mean information is outside the GPU REML path")
    if optimizer == "strict" and (G > 1 or residual_diag_stack is not None):
        # Strict likelihood comparisons need accurate solves (reml.py:1388-1408).
        pcg_tol = min(pcg_tol, 1e-5)
    t_start = time.time()
    full_log = bool(verbose) and log_detail == "full"

    base = int(seed) + 2026
    use_trace_probes = optimizer == "smile_scoring"
    n_trace = n_rand_vec if use_trace_probes else 0
    if use_trace_probes:
        Vrand = (trace_probes.to(dev, torch.float32) if trace_probes is not None
                 else rademacher(n, n_rand_vec, base * 3 + 1, dev))
    else:
        Vrand = None
    key_slq = base * 3 + 2

    if response_is_standardized:
        if not bool(torch.all(torch.isfinite(y))):
            raise ValueError("Phenotype contains non-finite values.")
        y_mean, y_scale = 0.0, 1.0
    else:
        y, ym, ys = standardize_response(y)
        y_mean, y_scale = float(ym), float(ys)

    xmat = None if covar is None else torch.as_tensor(covar, dtype=torch.float32).to(dev)
    if xmat is not None and xmat.numel() == 0:
        xmat = None
    if xmat is not None:
        if xmat.ndim == 1:
            xmat = xmat[:, None]
        if xmat.ndim != 2 or xmat.shape[0] != n:
            raise ValueError("covar must be a 2D matrix with one row per phenotype sample.")
        if not bool(torch.all(torch.isfinite(xmat))):
            raise ValueError("covar contains non-finite values.")
        if xmat.shape[1] >= n:
            raise ValueError("covar must have fewer columns than samples for REML.")
        _validate_fixed_effect_design(xmat)
        xmat = xmat.contiguous()

    if param_init is not None:
        p0 = np.asarray(param_init, dtype=np.float64).reshape(-1)
        if p0.size != G + E:
            raise ValueError(f"param_init length mismatch: expected {G + E}, got {p0.size}")
        if not np.all(np.isfinite(p0)):
            raise ValueError("param_init contains non-finite values.")
        tg0 = np.maximum(p0[:G], 0.0)
        tg0 = np.where(tg0 <= genetic_zero_tol, 0.0, tg0)
        param = np.concatenate([tg0, np.maximum(p0[G:], residual_floor)])
    else:
        gsum = float(np.sum(genetic_atoms))
        if not math.isfinite(gsum) or gsum <= 0.0:
            raise ValueError("At least one genetic component must have positive average diagonal.")
        rsum = float(np.sum(residual_atoms))
        if not math.isfinite(rsum) or rsum <= 0.0:
            raise ValueError("Residual components must have positive total average diagonal.")
        tg = np.where(genetic_atoms > 0.0, h2_init / gsum, 0.0)
        te = np.full(E, (1.0 - h2_init) / rsum)
        param = np.concatenate([np.maximum(tg, 0.0), np.maximum(te, residual_floor)])

    diag_atoms = None
    diag_stack = None
    if precond_conf is None or getattr(precond_conf, "diag_mode", None) != "scalar_identity":
        diag_atoms = _scalar_diag_from_diag_list(diag_list)
        if diag_atoms is None:
            diag_stack = torch.stack([
                torch.as_tensor(d, dtype=torch.float32).reshape(-1).to(dev).expand(n)
                if torch.as_tensor(d).ndim == 0 else torch.as_tensor(d, dtype=torch.float32).to(dev)
                for d in diag_list])

    KVrand, affine = _probe_setup(probe_cache, K_mvs, n, seed=seed, Vrand=Vrand,
                                  slq_samples=slq_samples, slq_m=slq_m,
                                  residual_free=residual_diag_stack is None, E=E,
                                  stacked_kv=stacked_kv, slq_probes=slq_probes, dev=dev)
    slq_probes_t = None if slq_probes is None else torch.as_tensor(slq_probes, dtype=torch.float32).to(dev)

    if slq_precond_conf is None:
        slq_precond_conf = precond_conf
    slq_ref = None
    if (slq_mode == "projected_core_residual" and affine is None and slq_precond_conf is not None
            and getattr(slq_precond_conf, "diag_mode", None) == "scalar_identity"
            and getattr(slq_precond_conf, "total_rank", 0) > 0):
        tgp = torch.as_tensor(param[:G], dtype=torch.float32, device=dev)
        tep = torch.as_tensor(param[G:], dtype=torch.float32, device=dev)
        ref_diag = scalar_diag_from_precond_conf(slq_precond_conf, tgp, tep)
        if ref_diag is None:
            raise ValueError("projected_core_residual SLQ requires a scalar-identity reference.")
        slq_ref = build_projected_core_runtime(slq_precond_conf, tgp, ref_diag, eps=precond_eps,
                                               need_invsqrt=True)
        if slq_ref is None:
            raise RuntimeError("Failed to build the fixed projected-core SLQ reference.")

    parts = []
    x_cols = 0
    if xmat is not None and xmat.shape[1] > 0:
        x_cols = xmat.shape[1]
        parts.append(xmat)
    y_col = x_cols
    parts.append(y[:, None])
    rand_stop = x_cols + 1 + n_trace
    if use_trace_probes:
        parts.append(Vrand)
    rhs_const = torch.cat(parts, dim=1).contiguous()

    ctx = REMLContext(
        n=n, G=G, E=E, K_mvs=K_mvs, weighted_hv=weighted_hv, stacked_kv=stacked_kv,
        diag_stack=diag_stack, residual_diag_stack=residual_diag_stack, xmat=xmat, y=y,
        rhs_const=rhs_const, y_col=y_col, rand_stop=rand_stop, n_XyZ_cols=rand_stop,
        R_rand=n_trace, kvrand_stack=KVrand, precond_conf=precond_conf, diag_atoms=diag_atoms,
        residual_diag_atoms=residual_atoms, affine_slq_cache=affine, slq_reference_runtime=slq_ref,
        slq_workspace_bytes=int(slq_workspace_bytes), slq_probes=slq_probes_t,
    )
    warm_all = torch.full_like(rhs_const, float("nan"))
    warm_ai = torch.full((n, G + E), float("nan"), dtype=torch.float32, device=dev)

    def run_eval(pvec, warm, wai, wr, war, taylor=None, *, compute_traces=use_trace_probes,
                 min_loglik=None):
        return _eval_once(ctx, pvec, warm, warm_ai=wai, key_slq=key_slq, minq_tol=pcg_tol,
                          maxiter=maxiter, precond_eps=precond_eps, slq_samples=slq_samples,
                          slq_m=slq_m, slq_mode=slq_mode, warm_ready=wr, warm_ai_ready=war,
                          taylor_logdet=taylor, compute_traces=compute_traces,
                          min_loglik=min_loglik)

    ll, grad, FI, k0, warm_all, warm_ai, trR, trK, logdet_c = run_eval(param, warm_all, warm_ai,
                                                                         False, False)
    if not (math.isfinite(ll) and np.all(np.isfinite(grad)) and np.all(np.isfinite(FI.mat))):
        raise FloatingPointError("Non-finite warmup state (ll/grad/FI).")
    stop_reason = "max_iter"
    history: list[dict] = []
    n_evals = 1
    for it in range(minq_iter):
        t_it = time.time()
        accepted = False
        alpha_try = 1.0
        ls_trace = []
        evaluated = 0
        last_err = None
        trial_count = 0
        ll_new, grad_new, FI_new = ll, grad, FI
        warm_next, warm_ai_next = warm_all, warm_ai
        trR_new, trK_new, logdet_new = trR, trK, logdet_c
        k_pcg = 0
        delta = np.zeros_like(param)
        upd = param
        max_rel_dp = 0.0
        use_taylor = False
        freeze = np.zeros(G, dtype=bool)
        step_norm = 0.0
        step_sec = eval_sec = 0.0
        eval_ai_pcg = 0
        step_stats = FisherSolveStats(free_dim=int(param.size)).to_dict()
        limit = 1 if optimizer == "smile_scoring" else max_linesearch_trials
        while trial_count < limit:
            trial_count += 1
            alpha_used = alpha_try
            t_step = time.perf_counter()
            step_dir, freeze = _projected_fisher_direction(
                param, grad, FI, n_genetic=G, genetic_zero_tol=genetic_zero_tol,
                residual_floor=residual_floor, trial_alpha=alpha_used)
            step_sec += time.perf_counter() - t_step
            n_frozen = int(np.sum(freeze))
            step_stats = (FI.stats.to_dict() if FI.stats is not None else FisherSolveStats(
                free_dim=int(param.size) - n_frozen, frozen_genetic=n_frozen).to_dict())
            upd, delta = _apply_projected_step(param, step_dir, alpha_used, n_genetic=G,
                                               genetic_zero_tol=genetic_zero_tol,
                                               residual_floor=residual_floor)
            step_norm = float(np.linalg.norm(delta))
            max_rel_dp = float(np.max(np.abs(delta) / np.maximum(np.abs(param), 1e-8)))
            taylor = None
            trial_taylor = False
            if optimizer == "smile_scoring" and max_rel_dp < taylor_threshold and logdet_c is not None:
                taylor = logdet_c + torch.dot(torch.as_tensor(delta[:G], dtype=torch.float64, device=dev), trK) \
                    + torch.dot(torch.as_tensor(delta[G:], dtype=torch.float64, device=dev), trR)
                trial_taylor = True
            t_eval = time.time()
            try:
                res = run_eval(upd, warm_all, warm_ai, True, True, taylor, compute_traces=False,
                               min_loglik=ll if optimizer == "strict" else None)
                n_evals += 1
            except FloatingPointError as err:
                eval_sec += time.time() - t_eval
                if optimizer == "smile_scoring":
                    raise
                last_err = err
                ls_trace.append((alpha_used, float("-inf"), False, 0, 0, False))
                alpha_try *= 0.5
                continue
            eval_sec += time.time() - t_eval
            ll_try, grad_try, FI_try, k_try, warm_try, wai_try, _, _, ld_try = res
            dll = ll_try - ll
            evaluated += 1
            ai_it = FI_try.stats.ai_pcg_iters if FI_try is not None and FI_try.stats else 0
            eval_ai_pcg = int(ai_it)
            ok = dll >= 0.0 or optimizer == "smile_scoring"
            ls_trace.append((alpha_used, dll, ok, k_try, ai_it, trial_taylor))
            if ok:
                accepted = True
                ll_new, grad_new, FI_new = ll_try, grad_try, FI_try
                warm_next, warm_ai_next = warm_try, wai_try
                if use_trace_probes:
                    trR_new, trK_new = _compute_traces_from_pcg(warm_try, ctx)
                logdet_new = ld_try
                k_pcg = k_try
                use_taylor = trial_taylor
                break
            alpha_try *= 0.5
        if evaluated == 0:
            raise FloatingPointError(
                f"REML line search could not evaluate any of {trial_count} candidates at "
                f"iteration {it + 1}: {last_err}") from last_err
        dll = ll_new - ll
        rel = dll / max(abs(ll), 1e-12)
        if accepted:
            if optimizer == "smile_scoring":
                stop = (not math.isfinite(rel)) or max_rel_dp < scoring_step_tol
            else:
                stop = (not math.isfinite(rel)) or rel < rel_dll_tol
        else:
            stop = True
        refreshed = False
        if accepted and not stop and (it + 1) < minq_iter and precond_refresh_fn is not None:
            new_conf = precond_refresh_fn(upd)
            if new_conf is None:
                raise RuntimeError("PCG preconditioner refresh returned no configuration.")
            ctx.precond_conf = new_conf
            refreshed = True
        history.append({
            "iter": it + 1,
            "status": ("accept" if dll >= 0 else "accept_downhill") if accepted else "ll_down",
            "accepted": accepted,
            "converged": bool(stop),
            "grad_norm": float(np.linalg.norm(grad_new)),
            "loglik": float(ll_new),
            "loglik_prev": float(ll),
            "dll_true": float(dll),
            "rel_dll": float(rel),
            "pcg_iters": int(k_pcg),
            "pcg_tol": pcg_tol,
            "step_norm": step_norm,
            "step_sec": step_sec,
            "step_alpha": alpha_used,
            "line_search_trials": trial_count,
            "line_search_trace": [
                {"alpha": a, "dll": d, "accepted": o, "pcg_iters": p, "ai_pcg_iters": q,
                 "used_taylor": t} for a, d, o, p, q, t in ls_trace],
            "n_freeze": int(np.sum(freeze)),
            "eval_ai_pcg_iters": eval_ai_pcg,
            "eval_sec": eval_sec,
            "iter_sec": time.time() - t_it,
            "params": [float(v) for v in (upd if accepted else param)],
            "slq_taylor": use_taylor,
            "max_rel_dp": max_rel_dp,
            "pcg_precond_refreshed": refreshed,
            "y_mean": y_mean,
            "y_scale": y_scale,
            **step_stats,
        })
        if full_log:
            logger.info("[REML] iter %d ll %.6e -> %.6e dll=%.3e alpha=%.3g ls=%d pcg=%d",
                        it + 1, ll, ll_new, dll, alpha_used, trial_count, k_pcg)
        if accepted:
            param, grad, FI, ll = upd, grad_new, FI_new, ll_new
            warm_all, warm_ai = warm_next, warm_ai_next
            trR, trK, logdet_c = trR_new, trK_new, logdet_new
            if stop:
                stop_reason = "scoring_step" if optimizer == "smile_scoring" else "rel_dll"
                break
        else:
            stop_reason = "ll_down"
            break
    if history:
        history[-1]["stop_reason"] = stop_reason
        history[-1]["n_evals"] = n_evals
    if verbose:
        logger.info("[REML] done elapsed=%.1fs stop=%s", time.time() - t_start, stop_reason)
    if return_diagnostics:
        diag = {"theta": param, "grad": grad, "ai": FI.mat, "loglik": ll,
                "stop_reason": stop_reason, "y_mean": y_mean, "y_scale": y_scale,
                "n_evals": n_evals,
                "logdet": None if logdet_c is None else float(logdet_c)}
        if use_trace_probes and trK is not None:
            # Hutchinson traces tr(H^-1 K_i), tr(H^-1 R_j) of the last accepted solve.
            diag["trace_K"] = torch.as_tensor(trK).double().cpu().numpy()
            diag["trace_R"] = torch.as_tensor(trR).double().cpu().numpy()
        if not unit_variance_components:
            diag["genetic_trace_atoms"] = genetic_atoms
            diag["residual_trace_atoms"] = residual_atoms
        return param, history, diag
    return param, history


__all__ = ["fit_reml", "standardize_response", "REMLProbeCache", "AffineSLQCache",
           "prime_probe_cache"]
