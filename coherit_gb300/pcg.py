"""Block preconditioned conjugate gradient (multi-RHS) on the GPU.

Same contract as GPU_REML's ``pcg_solve`` (pcg.py:68-167): every right-hand
side is scaled by an independent power of two, zero columns have the exact
solution zero, the recursive residual is checked every ``check_every``
iterations, and the returned relative residual is the verified true residual
``||B - H X|| / ||B||`` (maximum over columns); a failed verification
restarts from the true residual inside the same iteration budget.

The n x k vector work runs in the library's fused kernels: FP64 column
reductions and the fused X/R and P updates (pcg.py:31-65); only the per-
column scalars of a convergence check cross to the host.
"""
from __future__ import annotations

import math
from typing import Callable, Optional, Tuple

import torch

from . import _lib


def _identity(v):
    return v


def _cols(A: torch.Tensor) -> torch.Tensor:
    return A if A.ndim == 2 else A[:, None]


def coldot(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """Column sums of A*B in FP64 (device)."""
    A2, B2 = _cols(A), _cols(B)
    n, k = A2.shape
    out = torch.empty(k, dtype=torch.float64, device=A2.device)
    _lib.check(_lib.load().coherit_colreduce(
        0, n, k, A2.data_ptr(), A2.stride(0), B2.data_ptr(), B2.stride(0), out.data_ptr(),
        _lib.stream_ptr()), "column dot")
    return out


def colnorm2(A: torch.Tensor) -> torch.Tensor:
    """Column sums of squares in FP64 (device)."""
    A2 = _cols(A)
    n, k = A2.shape
    out = torch.empty(k, dtype=torch.float64, device=A2.device)
    _lib.check(_lib.load().coherit_colreduce(
        1, n, k, A2.data_ptr(), A2.stride(0), A2.data_ptr(), A2.stride(0), out.data_ptr(),
        _lib.stream_ptr()), "column norm")
    return out


def _pcg_state_update(X, R, P, rs, AP, active, breakdown):
    """X += P alpha, R -= AP alpha with alpha = rs / sum(P*AP) on valid active columns."""
    denom = coldot(P, AP)
    n, k = X.shape
    _lib.check(_lib.load().coherit_pcg_state_update(
        n, k, X.data_ptr(), X.stride(0), R.data_ptr(), R.stride(0), P.data_ptr(), P.stride(0),
        AP.data_ptr(), AP.stride(0), rs.data_ptr(), denom.data_ptr(), active.data_ptr(),
        breakdown.data_ptr(), _lib.stream_ptr()), "pcg state update")
    return X, R, breakdown


def _pcg_direction_update(P, R_new, Z_new, rs_old, threshold, active, rnorm):
    """P = active ? Z + beta P : 0 with the new residual norms (in place)."""
    rs_new = coldot(R_new, Z_new)
    rn2 = colnorm2(R_new)
    n, k = P.shape
    _lib.check(_lib.load().coherit_pcg_direction_update(
        n, k, P.data_ptr(), P.stride(0), Z_new.data_ptr(), Z_new.stride(0), rs_new.data_ptr(),
        rn2.data_ptr(), rs_old.data_ptr(), threshold.data_ptr(), active.data_ptr(),
        rnorm.data_ptr(), _lib.stream_ptr()), "pcg direction update")
    return P, rs_old, rnorm, active


def _as_matrix(B) -> torch.Tensor:
    if not isinstance(B, torch.Tensor):
        B = torch.as_tensor(B)
    return B


def pcg_solve(
    Hv: Callable,
    B,
    M: Optional[Callable] = None,
    tol: float = 1e-2,
    maxiter: int = 200,
    X0=None,
    check_every: int = 2,
) -> Tuple[torch.Tensor, torch.Tensor, int]:
    """Solve H X = B with block PCG; returns (X, max_rel_res, iters)."""
    if M is None:
        M = _identity
    check_every = max(1, int(check_every))
    B = _as_matrix(B)
    if B.device.type != "cuda":
        raise RuntimeError("pcg_solve runs on CUDA tensors (no CPU fallback)")
    B = B.to(torch.float32)
    vec = B.ndim == 1
    B2 = (B[:, None] if vec else B).contiguous()
    n, k = B2.shape
    dev = B2.device

    def shaped(A):
        return A[:, 0] if vec else A

    def apply(fn, A):
        out = fn(shaped(A))
        out = _as_matrix(out).to(device=dev, dtype=torch.float32)
        out = out[:, None] if out.ndim == 1 else out
        return out.contiguous()

    magnitude = B2.abs().amax(dim=0) if n > 0 else torch.zeros(k, device=dev)
    nonzero = magnitude > 0
    _, exponent = torch.frexp(magnitude)
    rhs_scale = torch.where(nonzero, torch.ldexp(torch.ones_like(magnitude), exponent - 1),
                            torch.ones_like(magnitude))
    Bs = (B2 / rhs_scale).contiguous()
    b_norm = torch.where(nonzero, colnorm2(Bs).sqrt(), torch.ones(k, dtype=torch.float64, device=dev))
    threshold = (tol * b_norm).contiguous()
    if X0 is None:
        solution = torch.zeros_like(B2)
    else:
        X0t = _as_matrix(X0).to(device=dev, dtype=torch.float32)
        X0t = X0t[:, None] if X0t.ndim == 1 else X0t
        solution = torch.where(nonzero[None, :], X0t, torch.zeros_like(X0t)).contiguous()

    def true_residual(value):
        residual = ((B2 - apply(Hv, value)) / rhs_scale).contiguous()
        norms = colnorm2(residual).sqrt()
        relative = torch.max(norms / b_norm)
        rel_host = float(relative)
        if not math.isfinite(rel_host):
            raise FloatingPointError("Non-finite true residual in PCG.")
        return residual, norms, relative, rel_host

    R, rnorm, res_final, rel_host = true_residual(solution)
    if rel_host <= tol or maxiter <= 0:
        return shaped(solution), res_final, 0

    def restart(sol, Rv, rn):
        X = (sol / rhs_scale).contiguous()
        active = (rn > threshold).to(torch.uint8)
        Z = apply(M, Rv)
        P = torch.where(active.bool()[None, :], Z, torch.zeros_like(Z)).contiguous()
        rs = torch.where(active.bool(), coldot(Rv, Z), torch.zeros(k, dtype=torch.float64, device=dev))
        return X, active.contiguous(), P, rs.contiguous()

    X, active, P, rs = restart(solution, R, rnorm)
    rnorm = rnorm.clone().contiguous()
    breakdown = torch.zeros(1, dtype=torch.int32, device=dev)
    it = 0
    while it < maxiter:
        AP = apply(Hv, P)
        X, R, breakdown = _pcg_state_update(X, R, P, rs, AP, active, breakdown)
        del AP
        Z = apply(M, R)
        P, rs, rnorm, active = _pcg_direction_update(P, R, Z, rs, threshold, active, rnorm)
        del Z
        it += 1
        if it % check_every == 0 or it == maxiter:
            recursive = float(torch.where(breakdown[0] != 0,
                                          torch.tensor(math.inf, dtype=torch.float64, device=dev),
                                          torch.max(rnorm / b_norm)))
            if not math.isfinite(recursive):
                raise FloatingPointError(
                    "PCG encountered nonpositive curvature or a non-finite recurrence."
                )
            if recursive <= tol or it == maxiter:
                solution = (X * rhs_scale).contiguous()
                R, rnorm, res_final, rel_host = true_residual(solution)
                if rel_host <= tol or it == maxiter:
                    return shaped(solution), res_final, it
                X, active, P, rs = restart(solution, R, rnorm)
                rnorm = rnorm.clone().contiguous()
    solution = (X * rhs_scale).contiguous()
    return shaped(solution), res_final, it


__all__ = ["pcg_solve", "coldot", "colnorm2"]
