"""SMILE block-weighted GRM in FP64 (test infrastructure only).

Restates smile_block_w.py's kernel ``K = sum_b Z_b W_b Z_b^T / c`` on
explicitly decoded, standardised genotypes (missing -> mean, i.e. 0 after
centring):

* per-block diagonal ``diag(Z_b W_b Z_b^T)`` and kernel trace per sample
  ``tr(Z_b W_b Z_b^T)/n`` (smile_block_w.py:669-716);
* the global normaliser c = sum of the blocks' trace contributions, either
  kernel traces or effective ranks (smile_block_w.py:718-726, :635-666);
* K V, one block's contribution, theta_e V + theta_g K V, and the SNP
  effects theta_g/c W_b Z_b^T alpha (smile_block_w.py:786-949);
* the multi-GRM weighted product sum_i theta_i K_i V + theta_e V
  (smile_block_w.py:1067-1104).

Blocks are (start, W) pairs with W None for the identity.
"""
from __future__ import annotations

import numpy as np

from .geno import diff_f64


def standardized(codes, mean, inv) -> np.ndarray:
    """Z (n, m) in FP64: (g - mean) * inv_sd, 0 where missing."""
    return diff_f64(codes, mean) * np.asarray(inv, dtype=np.float64)[None, :]


def standardized_fp32(codes, mean, inv) -> np.ndarray:
    """The reference's FP32 extraction: (g_imp - mean) * inv evaluated in FP32
    with missing imputed to the mean (geno_stream.py:2498-2501)."""
    g = codes.astype(np.float32)
    mean = np.asarray(mean, dtype=np.float32)[None, :]
    inv = np.asarray(inv, dtype=np.float32)[None, :]
    g_imp = np.where(codes == 3, mean, g)
    return ((g_imp - mean).astype(np.float32) * inv).astype(np.float32)


class SmileKernel:
    def __init__(self, Z: np.ndarray, blocks, *, normalization="kernel_trace",
                 effective_ranks=None):
        self.Z = np.asarray(Z, dtype=np.float64)
        self.blocks = [(int(s), None if W is None else np.asarray(W, dtype=np.float64))
                       for s, W in blocks]
        n = self.Z.shape[0]
        self.block_diag = []
        traces = []
        for i, (s, W) in enumerate(self.blocks):
            w = self._width(i)
            Zb = self.Z[:, s:s + w]
            d = np.sum(Zb * Zb, axis=1) if W is None else np.sum((Zb @ W) * Zb, axis=1)
            self.block_diag.append(d)
            if normalization == "effective_rank":
                traces.append(float(w) if effective_ranks is None else float(effective_ranks[i]))
            else:
                traces.append(float(d.sum()) / n)
        self.c = float(np.sum(traces))
        self.kernel_trace_total = float(sum(d.sum() for d in self.block_diag)) / n

    def _width(self, i):
        s, W = self.blocks[i]
        return self.sizes[i] if W is None else W.shape[0]

    @classmethod
    def identity(cls, Z, block_size, **kw):
        m = Z.shape[1]
        starts = list(range(0, m, block_size))
        obj = cls.__new__(cls)
        obj.sizes = [min(block_size, m - s) for s in starts]
        cls.__init__(obj, Z, [(s, None) for s in starts], **kw)
        return obj

    def diag_full(self) -> np.ndarray:
        return np.sum(self.block_diag, axis=0) / self.c

    def diag_mean(self) -> float:
        return self.kernel_trace_total / self.c

    def scores(self, XtV, block_idx=None, scale=1.0):
        out = np.zeros_like(XtV)
        for i, (s, W) in enumerate(self.blocks):
            if block_idx is not None and i != block_idx:
                continue
            w = self._width(i)
            local = XtV[s:s + w] if W is None else W @ XtV[s:s + w]
            out[s:s + w] += scale * local / self.c
        return out

    def kv(self, V, block_idx=None):
        V = np.asarray(V, dtype=np.float64)
        return self.Z @ self.scores(self.Z.T @ V, block_idx)

    def weighted_hv(self, theta_g, theta_e, V):
        V = np.asarray(V, dtype=np.float64)
        return float(theta_g) * self.kv(V) + (0.0 if theta_e is None else float(theta_e)) * V

    def snp_effects(self, alpha, theta_g):
        a = np.asarray(alpha, dtype=np.float64).reshape(-1, 1)
        return self.scores(self.Z.T @ a, scale=float(theta_g))[:, 0]

    def dense(self) -> np.ndarray:
        return self.kv(np.eye(self.Z.shape[0]))


def multi_weighted_hv(kernels, theta_g, theta_e, V):
    V = np.asarray(V, dtype=np.float64)
    out = sum(float(t) * k.kv(V) for t, k in zip(theta_g, kernels))
    return out + (0.0 if theta_e is None else float(theta_e)) * V
