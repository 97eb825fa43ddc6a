"""Projected-core preconditioner restated in numpy (test infrastructure only).

Follows precond.py:42-276 of the reference: M = d I + U C U^T with the
inverse / inverse square root on the projected subspace, its log-determinant
and the two-pass Nystrom basis.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg as sla


@dataclass
class Conf:
    U: np.ndarray
    core_atoms: np.ndarray
    total_rank: int
    n_grm: int
    diag_atoms: np.ndarray | None = None
    residual_diag_atoms: np.ndarray | None = None


@dataclass
class Runtime:
    U: np.ndarray
    total_rank: int
    d: float
    chol: np.ndarray
    eigvals: np.ndarray | None = None
    eigvecs: np.ndarray | None = None


def scalar_diag(conf: Conf, theta_g, theta_e) -> float:
    """precond.py:96-118"""
    da = np.ones(conf.n_grm) if conf.diag_atoms is None else np.asarray(conf.diag_atoms, float)
    te = np.asarray(theta_e, float).reshape(-1)
    ra = np.ones(te.size) if conf.residual_diag_atoms is None else np.asarray(conf.residual_diag_atoms, float)
    return float(te @ ra + np.asarray(theta_g, float) @ da)


def runtime(conf: Conf, theta_g, diag_H, eps=0.0, need_invsqrt=False) -> Runtime:
    """precond.py:121-171"""
    core = np.tensordot(np.asarray(theta_g, float), conf.core_atoms, axes=1)
    core = 0.5 * (core + core.T)
    d = max(float(diag_H) + eps, 1e-8)
    middle = core + d * np.eye(conf.total_rank)
    chol = np.linalg.cholesky(middle)
    ev = vec = None
    if need_invsqrt:
        ev, vec = np.linalg.eigh(middle)
        ev = np.clip(ev, 1e-8, None)
    return Runtime(conf.U, conf.total_rank, d, chol, ev, vec)


def apply_inverse(rt: Runtime, v):
    """precond.py:42-58"""
    rhs = rt.U.T @ v
    z = sla.cho_solve((rt.chol, True), rhs)
    return v / rt.d + rt.U @ (z - rhs / rt.d)


def apply_invsqrt(rt: Runtime, v):
    """precond.py:61-84"""
    rhs = rt.U.T @ v
    coeff = rt.eigvecs.T @ rhs
    vv = coeff / np.sqrt(np.clip(rt.eigvals, 1e-8, None))[:, None] if coeff.ndim == 2 else \
        coeff / np.sqrt(np.clip(rt.eigvals, 1e-8, None))
    z = rt.eigvecs @ vv
    s = 1.0 / np.sqrt(rt.d)
    return s * v + rt.U @ (z - s * rhs)


def logdet(rt: Runtime, n: int) -> float:
    """precond.py:207-221"""
    return (n - rt.total_rank) * np.log(rt.d) + 2.0 * np.sum(
        np.log(np.clip(np.diag(rt.chol), np.finfo(float).tiny, None)))


def lowrank_basis(K_mv, omega: np.ndarray, max_rank: int):
    """Nystrom basis from a given Gaussian test matrix (precond.py:251-276)."""
    Y = K_mv(omega)
    Q, _ = np.linalg.qr(Y, mode="reduced")
    Z = K_mv(Q)
    B = Q.T @ Z
    ev, vec = np.linalg.eigh(B)
    idx = np.argsort(ev)[::-1]
    ev = np.maximum(ev[idx], 0.0)
    vec = vec[:, idx]
    U = Q @ vec
    k = min(max_rank, U.shape[1])
    return U[:, :k], ev[:k]
