"""Block PCG restated in numpy FP32 (test infrastructure only).

Follows pcg.py:68-167 of the reference: independent power-of-two scaling of
every right-hand side (pcg.py:103-110), masked block recurrence with per-
column active flags (pcg.py:31-65), recursive convergence checks every
``check_every`` iterations (pcg.py:146-155), verification of the true
residual and restart from it within the same iteration budget
(pcg.py:113-120, :155-167).  Returns (X, max_rel_res, iters).
"""
from __future__ import annotations

import math

import numpy as np


def _identity(v):
    return v


def _state_update(X, R, P, rs, AP, active):
    """X, R updates of one step (pcg.py:31-48)."""
    denom = np.sum(P * AP, axis=0, dtype=np.float32)
    with np.errstate(invalid="ignore", over="ignore"):
        valid = (rs > 0) & (denom > 0) & np.isfinite(rs) & np.isfinite(denom)
        moving = active & valid
        alpha = np.where(moving, rs / np.where(moving, denom, 1), 0).astype(np.float32)
    return (X + P * alpha).astype(np.float32), (R - AP * alpha).astype(np.float32), bool(
        np.any(active & ~valid))


def _direction_update(P, R_new, Z_new, rs_old, threshold):
    """New search direction (pcg.py:51-65)."""
    rs_new = np.sum(R_new * Z_new, axis=0, dtype=np.float32)
    rnorm_new = np.linalg.norm(R_new, axis=0).astype(np.float32)
    active = rnorm_new > threshold
    with np.errstate(invalid="ignore", over="ignore", divide="ignore"):
        beta = np.where(active, rs_new / np.where(rs_old > 0, rs_old, 1), 0).astype(np.float32)
        P_new = np.where(active, Z_new + P * beta, 0).astype(np.float32)
    return P_new, np.where(active, rs_new, 0).astype(np.float32), rnorm_new, active


def pcg_solve(Hv, B, M=None, tol=1e-2, maxiter=200, X0=None, check_every=2,
              state_update=None):
    if M is None:
        M = _identity
    state_update = state_update or _state_update
    check_every = max(1, int(check_every))
    B = np.asarray(B, dtype=np.float32)
    magnitude = np.max(np.abs(B), axis=0)
    nonzero = magnitude > 0
    _, exponent = np.frexp(magnitude)
    rhs_scale = np.where(nonzero, np.ldexp(np.ones_like(magnitude), exponent - 1), 1).astype(np.float32)
    b_norm = np.where(nonzero, np.linalg.norm(B / rhs_scale, axis=0), 1).astype(np.float32)
    threshold = (tol * b_norm).astype(np.float32)
    solution = np.zeros_like(B) if X0 is None else np.where(nonzero, np.asarray(X0, np.float32), 0).astype(np.float32)

    def true_residual(value):
        residual = ((B - np.asarray(Hv(value), np.float32)) / rhs_scale).astype(np.float32)
        norms = np.linalg.norm(residual, axis=0).astype(np.float32)
        relative = float(np.max(norms / b_norm))
        if not math.isfinite(relative):
            raise FloatingPointError("Non-finite true residual in PCG.")
        return residual, norms, relative

    R, rnorm, rel = true_residual(solution)
    if rel <= tol or maxiter <= 0:
        return solution, rel, 0
    X = (solution / rhs_scale).astype(np.float32)
    active = rnorm > threshold
    Z = np.asarray(M(R), np.float32)
    P = np.where(active, Z, 0).astype(np.float32)
    rs = np.where(active, np.sum(R * Z, axis=0, dtype=np.float32), 0).astype(np.float32)
    k = 0
    breakdown = False
    while k < maxiter:
        AP = np.asarray(Hv(P), np.float32)
        X, R, invalid = state_update(X, R, P, rs, AP, active)
        breakdown = breakdown or invalid
        Z = np.asarray(M(R), np.float32)
        P, rs, rnorm, active = _direction_update(P, R, Z, rs, threshold)
        k += 1
        if k % check_every == 0 or k == maxiter:
            recursive = math.inf if breakdown else float(np.max(rnorm / b_norm))
            if not math.isfinite(recursive):
                raise FloatingPointError(
                    "PCG encountered nonpositive curvature or a non-finite recurrence.")
            if recursive <= tol or k == maxiter:
                solution = (X * rhs_scale).astype(np.float32)
                R, rnorm, rel = true_residual(solution)
                if rel <= tol or k == maxiter:
                    return solution, rel, k
                X = (solution / rhs_scale).astype(np.float32)
                active = rnorm > threshold
                Z = np.asarray(M(R), np.float32)
                P = np.where(active, Z, 0).astype(np.float32)
                rs = np.where(active, np.sum(R * Z, axis=0, dtype=np.float32), 0).astype(np.float32)
    solution = (X * rhs_scale).astype(np.float32)
    return solution, rel, k
