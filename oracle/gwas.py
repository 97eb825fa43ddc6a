"""Marginal GWAS statistics in FP64 (test infrastructure only).

Restates the reference's Frisch-Waugh-Lovell per-SNP OLS (gwas.py:110-185)
on an explicit standardised genotype matrix Z (missing -> 0).  Pinned by
tests against a direct least-squares fit of y on [X, z_j] for every SNP.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg
import scipy.stats


def scan(Z, counts, inv_sd, y, X):
    Z = np.asarray(Z, np.float64)
    y = np.asarray(y, np.float64)
    X = np.asarray(X, np.float64)
    n = y.size
    Q, R, _ = scipy.linalg.qr(X, mode="economic", pivoting=True)
    d = np.abs(np.diag(R))
    tol = np.finfo(np.float64).eps * max(X.shape) * max(1.0, float(d.max()))
    rank = int(np.count_nonzero(d > tol))
    Q = Q[:, :rank]
    y_perp = y - Q @ (Q.T @ y)
    dof = n - rank - 1
    x_ty = Z.T @ y_perp
    x_var = np.asarray(counts, np.float64) - np.sum((Z.T @ Q) ** 2, axis=1)
    beta_std = x_ty / x_var
    rss = np.maximum(y_perp @ y_perp - beta_std * x_ty, 0.0)
    se_std = np.sqrt(rss / dof / x_var)
    t = beta_std / se_std
    p = 2.0 * scipy.stats.t.sf(np.abs(t), dof)
    inv = np.asarray(inv_sd, np.float64)
    return {"beta_std": beta_std, "se_std": se_std, "t": t, "p": p, "beta": beta_std * inv,
            "se": se_std * inv, "dof": dof}
