"""Rare-variant sparse ("sparse12") genotype operator (test infrastructure only).

Restates, in numpy, the reference's sparse path:

* the single-pass BED build: per-SNP het / hom-alt / missing counts and the
  FP32 statistics (sparse_stream.py:518-567, :711-742), then the per-SNP
  entry lists in sample order with values 1 (het), 2 (hom-alt) and 3
  (missing, imputed to the SNP mean when used) (sparse_stream.py:570-606);
* the shard payload: a0 = -mean*inv, b = a0*inv, inv_sq = inv^2,
  row_b = sum_j x_ij b_j and sum_a0_sq = sum_j a0_j^2
  (sparse_stream.py:1037-1145, :1282-1297);
* the operator ``K V = row_sparse + row_b sum_v + (sum_a0_sq sum_v + b.xtv)``
  (kv_impl.py:777-817), ``X^T V`` (kv_impl.py:752-774) and the projected-core
  atom (kv_impl.py:829-849), evaluated in FP64 by segment sums over the
  entries, normalised by m_eff (sparse_stream.py:1344-1388).

Parity of this restatement is pinned by tests against the dense FP64 oracle
(`oracle.geno.kv_f64` on the same genotype codes), which it must equal to
rounding.
"""
from __future__ import annotations

import numpy as np

from . import geno as og

HET, HOM, MISS = 1, 2, 3


def codes_from_bed(bed: bytes | np.ndarray, n_full: int, m: int, keep=None) -> np.ndarray:
    """(n_keep, m) allele counts 0/1/2 and 3 = missing from PLINK BED bytes.

    BED 2-bit codes 00, 01, 10, 11 are hom-A1 (2 copies), missing, het (1)
    and hom-A2 (0) (sparse_stream.py:540-555)."""
    raw = np.frombuffer(bytes(bed), dtype=np.uint8) if not isinstance(bed, np.ndarray) else bed
    if raw.size < 3 or raw[0] != 0x6C or raw[1] != 0x1B or raw[2] != 0x01:
        raise ValueError("not a SNP-major PLINK .bed")
    bps = (int(n_full) + 3) // 4
    body = raw[3:3 + bps * int(m)].reshape(int(m), bps)
    shifts = 2 * (np.arange(int(n_full)) % 4)
    two = (body[:, np.arange(int(n_full)) // 4] >> shifts[None, :]) & 3
    lut = np.array([2, 3, 1, 0], dtype=np.uint8)
    codes = lut[two].T
    if keep is not None:
        codes = codes[np.asarray(keep, dtype=np.int64)]
    return np.ascontiguousarray(codes)


def csc_from_codes(codes: np.ndarray):
    """Per-SNP entries in sample order: (col_off[m+1], rows[nnz], vals[nnz]),
    vals 1 = het, 2 = hom-alt, 3 = missing (sparse_stream.py:570-606)."""
    c = np.asarray(codes)
    n, m = c.shape
    nz_cols, nz_rows = np.nonzero(c.T != 0)   # column-major order, rows ascending
    counts = np.bincount(nz_cols, minlength=m)
    col_off = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(counts, out=col_off[1:])
    vals = c[nz_rows, nz_cols].astype(np.int8)
    return col_off, nz_rows.astype(np.int32), vals


def bed_counts_stats(codes: np.ndarray):
    """Het / hom / missing counts and the FP32 statistics of the single-pass
    build (sparse_stream.py:518-567, :711-742): cnt = non-missing samples,
    s1 = allele sum, s2 = squared allele sum, then the reference's separately
    rounded FP32 mean / inverse sd."""
    c = np.asarray(codes)
    n_het = (c == HET).sum(axis=0).astype(np.int64)
    n_hom = (c == HOM).sum(axis=0).astype(np.int64)
    n_miss = (c == MISS).sum(axis=0).astype(np.int64)
    cnt = c.shape[0] - n_miss
    s1 = n_het + 2 * n_hom
    s2 = n_het + 4 * n_hom
    mean, inv = og.fp32_stats(cnt, s1, s2)
    return {"n_het": n_het, "n_hom": n_hom, "n_miss": n_miss, "cnt": cnt, "mean": mean,
            "inv": inv, "eff": float(np.count_nonzero(inv > 0)),
            "atom": (float(np.sum(cnt[inv > 0], dtype=np.float64)
                           / (c.shape[0] * np.count_nonzero(inv > 0)))
                     if np.count_nonzero(inv > 0) else 0.0)}


def entry_values(col_off, vals, mean) -> np.ndarray:
    """FP64 value of every entry: 1, 2, or the SNP mean for a missing entry
    (kv_impl.py:746-749)."""
    cols = np.repeat(np.arange(col_off.size - 1), np.diff(col_off))
    v = vals.astype(np.float64)
    miss = vals == MISS
    v[miss] = np.asarray(mean, np.float64)[cols[miss]]
    return v, cols


def shard_payload(col_off, rows, vals, mean, inv, n: int) -> dict:
    """b, inv_sq, row_b and sum_a0_sq of one shard (sparse_stream.py:1037-1145)."""
    mean = np.asarray(mean, np.float64)
    inv = np.asarray(inv, np.float64)
    a0 = -mean * inv
    b = a0 * inv
    v, cols = entry_values(col_off, vals, mean)
    row_b = np.bincount(rows, weights=v * b[cols], minlength=n)
    return {"mean": mean, "inv": inv, "b": b, "inv_sq": inv * inv, "row_b": row_b,
            "sum_a0_sq": float(a0 @ a0), "a0": a0}


def xtv_f64(col_off, rows, vals, mean, inv, V) -> np.ndarray:
    """Standardised ``Z^T V`` (kv_impl.py:752-774)."""
    V = np.asarray(V, np.float64)
    squeeze = V.ndim == 1
    V = V[:, None] if squeeze else V
    v, cols = entry_values(col_off, vals, mean)
    m = col_off.size - 1
    xtv = np.zeros((m, V.shape[1]))
    np.add.at(xtv, cols, v[:, None] * V[rows])
    out = np.asarray(inv, np.float64)[:, None] * (xtv - np.asarray(mean, np.float64)[:, None]
                                                   * V.sum(axis=0)[None, :])
    return out[:, 0] if squeeze else out


def kv_f64(col_off, rows, vals, mean, inv, V, eff=None) -> np.ndarray:
    """``K V`` through the reference's shard decomposition (kv_impl.py:777-817),
    divided by m_eff when ``eff`` is given and positive."""
    V = np.asarray(V, np.float64)
    squeeze = V.ndim == 1
    V = V[:, None] if squeeze else V
    n = V.shape[0]
    p = shard_payload(col_off, rows, vals, mean, inv, n)
    v, cols = entry_values(col_off, vals, mean)
    m = col_off.size - 1
    sum_v = V.sum(axis=0)
    xtv = np.zeros((m, V.shape[1]))
    np.add.at(xtv, cols, v[:, None] * V[rows])
    weighted = p["inv_sq"][:, None] * xtv
    row_sparse = np.zeros((n, V.shape[1]))
    np.add.at(row_sparse, rows, v[:, None] * weighted[cols])
    base = p["sum_a0_sq"] * sum_v + p["b"] @ xtv
    out = row_sparse + p["row_b"][:, None] * sum_v[None, :] + base[None, :]
    if eff is not None and eff > 0:
        out = out / float(eff)
    return out[:, 0] if squeeze else out


def projected_core_atom_f64(col_off, rows, vals, mean, inv, U, eff, subtract_identity=True):
    """``(Z^T U)^T (Z^T U) / m_eff - I`` (kv_impl.py:829-849,
    sparse_stream.py:1423-1461)."""
    blk = xtv_f64(col_off, rows, vals, mean, inv, U)
    core = blk.T @ blk
    if eff <= 0:
        return np.zeros_like(core)
    core = core / float(eff)
    if subtract_identity:
        core = core - np.eye(core.shape[0])
    return core


def synth_maf_q24_range(seed: int, snps, lo_q24: int, hi_q24: int) -> np.ndarray:
    """Rare-variant MAF of each SNP on a 2^24 scale, uniform on [lo, hi)
    (the dense generator's per-SNP hash with another range)."""
    s = np.asarray(snps, dtype=np.uint64)
    U = np.uint64
    with np.errstate(over="ignore"):
        h = og._splitmix64(np.full(s.shape, seed, dtype=np.uint64) * U(0xD1B54A32D192ED03) + s)
    return (U(lo_q24) + (h >> U(20)) % U(hi_q24 - lo_q24)).astype(np.uint32)


def synth_rare_codes(seed: int, n: int, snps, lo_q24: int, hi_q24: int,
                     missing_q24: int = 0) -> np.ndarray:
    """Codes (samples x SNPs) of the device's rare-variant generator: the
    dense generator's per-(SNP, sample) hash with the MAF drawn from
    [lo, hi) / 2^24."""
    s = np.asarray(snps, dtype=np.uint64).reshape(-1)
    i = np.arange(n, dtype=np.uint64)
    U = np.uint64
    with np.errstate(over="ignore"):
        key_s = og._splitmix64(np.full(s.shape, seed, dtype=np.uint64) ^ (s * U(0x8CB92BA72F3D8DD7)))
        h = og._splitmix64(key_s[None, :] ^ (i[:, None] * U(0x9E3779B97F4A7C15)))
    maf = synth_maf_q24_range(seed, s, lo_q24, hi_q24).astype(np.uint64)[None, :]
    codes = ((h & U(0xFFFFFF)) < maf).astype(np.uint8) + (((h >> U(24)) & U(0xFFFFFF)) < maf)
    codes = codes.astype(np.uint8)
    if missing_q24:
        codes[((h >> U(48)) * U(256)) < U(missing_q24)] = MISS
    return codes


def rare_codes(seed: int, n: int, m: int, maf_lo: float = 0.0005, maf_hi: float = 0.02,
               missing: float = 0.0) -> np.ndarray:
    """Seeded rare-variant genotypes: MAF ~ U(maf_lo, maf_hi) per SNP,
    Binomial(2, MAF) per sample, optional missing rate."""
    rng = np.random.default_rng(seed)
    maf = rng.uniform(maf_lo, maf_hi, size=m)
    codes = rng.binomial(2, maf[None, :], size=(n, m)).astype(np.uint8)
    if missing > 0:
        codes[rng.random((n, m)) < missing] = MISS
    return codes
