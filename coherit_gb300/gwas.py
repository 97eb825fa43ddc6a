"""Continuous-trait marginal GWAS scan on the resident genotype matrix.

Per SNP j the OLS effect of the standardised genotype z_j on the phenotype
after projecting out the covariates (Frisch-Waugh-Lovell), as the reference
computes it (gwas.py:70-230):

    Q        orthonormal basis of the covariates (pivoted QR, rank-revealing)
    y_perp   y - Q Q^T y
    [x^T y_perp, x^T Q] = Z^T [y_perp | Q]        one X^T V pass on the device
    x_var    n_obs,j - ||Q^T z_j||^2
    beta_std = x^T y_perp / x_var,  rss = y_perp'y_perp - beta_std x^T y_perp
    se_std   = sqrt(rss / dof / x_var),  t = beta_std / se_std,  dof = n - rank - 1
    beta, se = beta_std, se_std scaled by inv_sd_j (allele-count scale)
    p        two-sided Student t

The per-SNP arithmetic runs in FP64 on the device; p-values come from
scipy's t distribution on the host.  Output: the reference's TSV columns and
metadata JSON (gwas_io.py:8-31).
"""
from __future__ import annotations

import dataclasses
import json
import logging
import os

import numpy as np
import scipy.linalg
import scipy.stats
import torch

logger = logging.getLogger(__name__)

GWAS_HEADER = (
    "component_index\tcomponent_name\tvariant_index_global\tvariant_index_local\t"
    "chrom\tvariant_id\tcm\tbp\ta1\ta2\taf\tn_obs\tbeta\tse\tbeta_std\tse_std\tt\tp\n"
)
_WRITE_CHUNK_ROWS = 8192


@dataclasses.dataclass(frozen=True)
class GWASSummary:
    out_path: str
    metadata_path: str
    n_samples: int
    n_variants: int
    dof: int
    n_covar_cols: int


def _orthonormal_covariate_basis(X: np.ndarray) -> tuple[np.ndarray, int]:
    """Rank-revealing orthonormal basis of the covariates (gwas.py:30-43)."""
    if X.ndim != 2:
        raise ValueError("Covariate matrix must be 2D.")
    if X.shape[1] == 0:
        return np.empty((X.shape[0], 0), dtype=np.float32), 0
    Q, R, _ = scipy.linalg.qr(X.astype(np.float64, copy=False), mode="economic", pivoting=True)
    diag = np.abs(np.diag(R))
    if diag.size == 0:
        return np.empty((X.shape[0], 0), dtype=np.float32), 0
    tol = np.finfo(np.float64).eps * max(X.shape) * max(1.0, float(diag.max()))
    rank = int(np.count_nonzero(diag > tol))
    if rank == 0:
        return np.empty((X.shape[0], 0), dtype=np.float32), 0
    return np.asarray(Q[:, :rank], dtype=np.float32), rank


def marginal_scan(streamer, y, covar=None) -> dict:
    """Per-SNP marginal statistics of one streamer; arrays of length m."""
    y_np = np.asarray(y, dtype=np.float32).reshape(-1)
    n = int(y_np.shape[0])
    if n != int(streamer.n):
        raise ValueError(f"Sample-size mismatch between phenotype (n={n}) and streamer "
                         f"(n={int(streamer.n)}).")
    if getattr(streamer, "_means_host", None) is None or \
            getattr(streamer, "_inv_sds_host", None) is None:
        raise ValueError("GWAS requires keep_host_stats=True on dense streamers.")
    if getattr(streamer, "_count_host", None) is None:
        raise ValueError("GWAS requires per-SNP non-missing counts; rebuild streamers without "
                         "standardization_override or with host stats retained.")
    if np.asarray(streamer._count_host).size != int(streamer.m):
        raise RuntimeError("Internal GWAS count vector length mismatch.")
    if covar is None or np.size(covar) == 0:
        X = np.ones((n, 1), dtype=np.float32)
    else:
        X = np.asarray(covar, dtype=np.float32)
        if X.ndim == 1:
            X = X[:, None]
        if X.shape[0] != n:
            raise ValueError(f"Covariate row mismatch: expected {n}, got {int(X.shape[0])}.")
    Q, rank = _orthonormal_covariate_basis(X)
    y_perp = y_np if rank == 0 else (y_np - Q @ (Q.T @ y_np)).astype(np.float32)
    y_perp_ss = float(np.dot(y_perp.astype(np.float64), y_perp.astype(np.float64)))
    dof = int(n - rank - 1)
    if dof <= 0:
        raise ValueError(f"GWAS degrees of freedom must be positive; got n={n}, "
                         f"rank(X)={rank}, dof={dof}.")
    V = np.concatenate([y_perp[:, None]] + ([Q] if rank > 0 else []), axis=1)
    cross = streamer.xtv(torch.as_tensor(np.ascontiguousarray(V), device=streamer.dev),
                         normalize=False).double()
    dev = cross.device
    x_ty = cross[:, 0]
    proj_ss = (cross[:, 1:] ** 2).sum(dim=1) if rank > 0 else torch.zeros_like(x_ty)
    counts = torch.as_tensor(np.asarray(streamer._count_host, np.float64), device=dev)
    inv_sd = torch.as_tensor(np.asarray(streamer._inv_sds_host, np.float64), device=dev)
    means = np.asarray(streamer._means_host, np.float64)
    x_var = counts - proj_ss
    valid = (inv_sd > 0) & (x_var > 1e-8)
    nan = torch.full_like(x_ty, float("nan"))
    beta_std = torch.where(valid, x_ty / torch.where(valid, x_var, 1.0), nan)
    rss = torch.clamp(y_perp_ss - beta_std * x_ty, min=0.0)
    se_std = torch.where(valid, torch.sqrt(rss / dof / torch.where(valid, x_var, 1.0)), nan)
    ok = valid & (se_std > 0)
    beta = torch.where(ok, beta_std * inv_sd, nan)
    se = torch.where(ok, se_std * inv_sd, nan)
    t = torch.where(ok, beta_std / torch.where(ok, se_std, 1.0), nan)
    t_h = t.cpu().numpy()
    p = np.full_like(t_h, np.nan)
    fin = np.isfinite(t_h)
    p[fin] = 2.0 * scipy.stats.t.sf(np.abs(t_h[fin]), dof)
    return {"beta": beta.cpu().numpy(), "se": se.cpu().numpy(),
            "beta_std": beta_std.cpu().numpy(), "se_std": se_std.cpu().numpy(), "t": t_h,
            "p": p, "af": means / 2.0, "n_obs": np.asarray(streamer._count_host),
            "dof": dof, "rank": rank, "n_covar_cols": int(X.shape[1])}


def _bim_records(prefix: str):
    with open(prefix + ".bim", encoding="utf-8") as f:
        for line_no, line in enumerate(f, start=1):
            cols = line.rstrip("\n").split()
            if not cols:
                continue
            if len(cols) < 6:
                raise ValueError(f"{prefix}.bim: line {line_no} has fewer than 6 fields.")
            yield cols[:6]


def run_continuous_gwas(fitter, y, covar=None, *, out_prefix: str) -> GWASSummary:
    """Scan every dense streamer of the fitter (fitters with rare-variant
    streamers are rejected, gwas.py:77-86) and write ``<out_prefix>.gwas.tsv``
    and ``<out_prefix>.gwas_metadata.json`` (gwas.py:70-230)."""
    if getattr(fitter, "_has_sparse", False):
        raise ValueError("GWAS currently supports dense genotype inputs only.")
    streamers = list(getattr(fitter, "streamers", ()))
    n_dense = getattr(fitter, "_n_dense_streamers", len(streamers))
    streamers = streamers[:n_dense]
    if not streamers:
        raise ValueError("GWAS requires at least one dense genotype streamer.")
    if not out_prefix:
        raise ValueError("GWAS output requires a non-empty out_prefix.")
    out_path = out_prefix + ".gwas.tsv"
    os.makedirs(os.path.dirname(out_path) or ".", exist_ok=True)
    n = int(np.asarray(y).reshape(-1).shape[0])
    total, global_idx = 0, 0
    names, counts = [], []
    meta = None
    with open(out_path, "w") as fh:
        fh.write(GWAS_HEADER)
        for ci, st in enumerate(streamers):
            prefix = getattr(st, "bed_prefix", None)
            if not prefix:
                raise ValueError("Unable to resolve variant metadata sidecar path for GWAS "
                                 "input; dense inputs need a BED .bim sidecar.")
            prefix = prefix[:-4] if prefix.endswith(".bed") else prefix
            name = os.path.basename(prefix)
            stats = marginal_scan(st, y, covar)
            meta = stats
            rows = []
            li = -1
            for li, rec in enumerate(_bim_records(prefix)):
                if li >= int(st.m):
                    break
                rows.append(
                    f"{ci}\t{name}\t{global_idx}\t{li}\t{rec[0]}\t{rec[1]}\t{rec[2]}\t{rec[3]}\t"
                    f"{rec[4]}\t{rec[5]}\t{stats['af'][li]:.8g}\t{int(stats['n_obs'][li])}\t"
                    f"{stats['beta'][li]:.8g}\t{stats['se'][li]:.8g}\t"
                    f"{stats['beta_std'][li]:.8g}\t{stats['se_std'][li]:.8g}\t"
                    f"{stats['t'][li]:.8g}\t{stats['p'][li]:.8g}\n")
                global_idx += 1
                if len(rows) >= _WRITE_CHUNK_ROWS:
                    fh.write("".join(rows))
                    rows.clear()
            fh.write("".join(rows))
            if li + 1 != int(st.m):
                raise RuntimeError(f"Variant metadata count mismatch for {name}: "
                                   f"expected {int(st.m)}, got {li + 1}.")
            total += int(st.m)
            names.append(name)
            counts.append(int(st.m))
    meta_path = out_prefix + ".gwas_metadata.json"
    with open(meta_path, "w") as f:
        json.dump({"trait_type": "continuous", "model": "marginal_ols_fwl", "n_samples": n,
                   "n_variants": total, "n_covar_cols": meta["n_covar_cols"],
                   "rank_covar": meta["rank"], "dof": meta["dof"], "files": {"gwas": out_path},
                   "components": [{"component_index": i, "component_name": nm, "n_variants": c}
                                  for i, (nm, c) in enumerate(zip(names, counts))]},
                  f, indent=2, sort_keys=True)
    return GWASSummary(out_path=out_path, metadata_path=meta_path, n_samples=n,
                       n_variants=total, dof=meta["dof"], n_covar_cols=meta["n_covar_cols"])


__all__ = ["GWASSummary", "GWAS_HEADER", "marginal_scan", "run_continuous_gwas"]
