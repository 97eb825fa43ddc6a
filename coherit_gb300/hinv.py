"""H^{-1} solves for the weighted-LASSO fixed-effect path on the GPU operator.

The sparse REML pipeline screens and fits fixed effects with
V^{-1} = H^{-1} applied to many columns (phenotype, covariates, candidate
genotype columns).  These are the solver-side pieces it calls, with the
reference's names and behaviour:

* ``solve_hinv_columns_batched`` -- H X = B in bounded right-hand-side
  batches, each a block PCG on the tensor-core operator, rejecting a batch
  whose verified relative residual exceeds 1.05 x tol
  (run_sparse_reml_pipeline.py:1202-1297);
* ``require_pcg_converged`` (run_sparse_reml_pipeline.py:1182-1198);
* ``compute_projected_hinv_vector`` -- P_C t = H^{-1}t - H^{-1}C (C^T H^{-1}C)^{-1}
  C^T H^{-1}t in FP64 (lasso_cd.py:791-822) with ``solve_spd``
  (pipeline_common.py:407-421).

Right-hand sides may be host arrays (results returned on the host, as the
reference does) or CUDA tensors (results stay on the device).  Batches of
<= 80 columns fill one tensor-core launch per PCG iteration at bf16x3.
"""
from __future__ import annotations

from typing import Callable

import numpy as np
import scipy.linalg as sla
import torch

from .pcg import pcg_solve


def require_pcg_converged(rel_res, *, tol: float, iters: int, maxiter: int, stage: str) -> float:
    """Reject statistics built from an unconverged PCG solve."""
    rel = float(torch.as_tensor(rel_res).double().max()) if not isinstance(rel_res, float) \
        else float(rel_res)
    if (not np.isfinite(rel)) or rel > float(tol) * 1.05:
        raise RuntimeError(
            f"{stage} PCG did not converge: relative residual={rel:.3e}, "
            f"tolerance={float(tol):.3e}, iterations={int(iters)}/{int(maxiter)}.")
    return rel


def solve_hinv_columns_batched(*, hv: Callable, precond: Callable | None, rhs, warm_start,
                               tol: float, maxiter: int, batch_size: int, stage: str):
    """Solve ``H X = B`` in batches of ``batch_size`` columns.

    Returns ``(X, diagnostics)``; ``X`` is a numpy array for host ``rhs`` and a
    CUDA tensor for device ``rhs``."""
    on_device = isinstance(rhs, torch.Tensor) and rhs.is_cuda
    B = rhs if on_device else np.asarray(rhs, dtype=np.float32)
    if B.ndim != 2:
        raise ValueError("Batched PCG right-hand side must be a matrix.")
    n_rows, n_columns = int(B.shape[0]), int(B.shape[1])
    batch = int(batch_size)
    if batch < 1:
        raise ValueError("Batched PCG size must be positive.")
    W = None
    if warm_start is not None:
        W = warm_start if on_device else np.asarray(warm_start, dtype=np.float32)
        if tuple(W.shape) != (n_rows, n_columns):
            raise ValueError("Batched PCG warm start does not align with RHS.")
        finite = bool(torch.isfinite(W).all()) if on_device else bool(np.all(np.isfinite(W)))
        if not finite:
            raise ValueError("Batched PCG warm start must be finite.")
    finite = bool(torch.isfinite(B).all()) if on_device else bool(np.all(np.isfinite(B)))
    if not finite:
        raise ValueError("Batched PCG right-hand side must be finite.")
    empty_diag = {"batch_size": batch, "n_batches": 0, "n_columns": 0,
                  "max_reported_relative_residual": 0.0, "max_true_relative_residual": 0.0,
                  "max_iterations": 0, "total_batch_iterations": 0}
    if n_columns == 0:
        out = (torch.empty((n_rows, 0), dtype=torch.float32, device=B.device) if on_device
               else np.empty((n_rows, 0), dtype=np.float32))
        return out, empty_diag
    dev = B.device if on_device else torch.device("cuda", torch.cuda.current_device())
    Bd = B.to(torch.float32) if on_device else torch.as_tensor(B, device=dev)
    Wd = None if W is None else (W.to(torch.float32) if on_device else torch.as_tensor(W, device=dev))
    X = torch.empty_like(Bd)
    max_rep, max_iter, total_iter, n_batches = 0.0, 0, 0, 0
    for start in range(0, n_columns, batch):
        stop = min(start + batch, n_columns)
        x0 = None if Wd is None else Wd[:, start:stop].contiguous()
        sol, rep, iters = pcg_solve(hv, Bd[:, start:stop].contiguous(), M=precond, tol=float(tol),
                                    maxiter=int(maxiter), X0=x0)
        rep = require_pcg_converged(rep, tol=float(tol), iters=int(iters), maxiter=int(maxiter),
                                    stage=f"{stage} columns {start}:{stop}")
        # pcg_solve reports the verified B - H X residual; no second pass.
        X[:, start:stop] = sol
        max_rep = max(max_rep, rep)
        max_iter = max(max_iter, int(iters))
        total_iter += int(iters)
        n_batches += 1
    diag = {"batch_size": batch, "n_batches": n_batches, "n_columns": n_columns,
            "max_reported_relative_residual": max_rep, "max_true_relative_residual": max_rep,
            "max_iterations": max_iter, "total_batch_iterations": total_iter}
    return (X if on_device else X.cpu().numpy()), diag


def solve_spd(mat: np.ndarray, rhs: np.ndarray, ridge: float = 0.0) -> np.ndarray:
    """FP64 Cholesky solve, falling back to a general solve."""
    A = np.asarray(mat, dtype=np.float64)
    B = np.asarray(rhs, dtype=np.float64)
    if A.ndim != 2 or A.shape[0] != A.shape[1]:
        raise ValueError("SPD solve expects a square matrix.")
    if A.shape[0] == 0:
        return np.zeros_like(B, dtype=np.float64)
    if ridge > 0.0:
        A = A + float(ridge) * np.eye(A.shape[0])
    try:
        L = sla.cholesky(A, lower=True, check_finite=False)
        return sla.solve_triangular(L.T, sla.solve_triangular(L, B, lower=True, check_finite=False),
                                    lower=False, check_finite=False)
    except np.linalg.LinAlgError:
        return np.linalg.solve(A, B)


def compute_projected_hinv_vector(covar, Hinv_covar, Hinv_target, ridge: float = 1e-6) -> np.ndarray:
    """``P_C t = H^{-1}t - H^{-1}C (C^T H^{-1} C)^{-1} C^T H^{-1} t`` in FP64."""
    t = np.asarray(Hinv_target, dtype=np.float64).reshape(-1)
    if covar is None or Hinv_covar is None or np.asarray(Hinv_covar).size == 0:
        return t
    C = np.asarray(covar, dtype=np.float64)
    HC = np.asarray(Hinv_covar, dtype=np.float64)
    if C.ndim != 2 or HC.ndim != 2:
        raise ValueError("covar/Hinv_covar must be 2D.")
    if C.shape != HC.shape:
        raise ValueError("covar and Hinv_covar shape mismatch.")
    if C.shape[0] != t.size:
        raise ValueError("Hinv_target length mismatch with covariates.")
    A = C.T @ HC
    if A.size > 0:
        A = 0.5 * (A + A.T) + float(ridge) * np.eye(A.shape[0])
    return t - HC @ solve_spd(A, C.T @ t)


__all__ = ["require_pcg_converged", "solve_hinv_columns_batched", "solve_spd",
           "compute_projected_hinv_vector"]
