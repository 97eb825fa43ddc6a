"""Genotype side of the oracle (test infrastructure only).

Restates, in numpy:

* the reference's 2-bit packed call-block cache (kv_impl.py:58-66,
  geno_stream.py:885-926, :1258-1264, :1323-1331) and its call geometry
  (geno_stream.py:469-505);
* the FP32 per-SNP statistics (geno_stream.py:1780-1792) and the
  mean-diagonal atoms (geno_stream.py:1409-1444, :1482-1503);
* the genotype operator ``sum_c Z_c Z_c^T V / m_eff`` (kv_impl.py:69-113,
  :268-326, :1042-1187), X^T V (kv_impl.py:163-185) and Z b
  (kv_impl.py:221-265) evaluated in FP64 on explicitly decoded genotypes;
* the FP32 streamed form of ``kv_impl_streamed`` (per call block: decode,
  impute, centre, two FP32 matmuls) which is timed as the CPU baseline;
* the exact diagonal (geno_stream.py:929-955, :2780-2821);
* the counter-based synthetic generator shared with the CUDA library.
"""
from __future__ import annotations

import numpy as np

MISSING = 3

# ------------------------------------------------------------------ generator

_U = np.uint64


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x + _U(0x9E3779B97F4A7C15)
        x = (x ^ (x >> _U(30))) * _U(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> _U(27))) * _U(0x94D049BB133111EB)
    return x ^ (x >> _U(31))


def synth_maf_q24(seed: int, snps: np.ndarray) -> np.ndarray:
    """MAF of each SNP on a 2^24 scale, uniform on [0.05, 0.5)."""
    s = np.asarray(snps, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = _splitmix64(np.full(s.shape, seed, dtype=np.uint64) * _U(0xD1B54A32D192ED03) + s)
    return (_U(838861) + (h >> _U(20)) % _U(7549747)).astype(np.uint32)


def synth_codes(seed: int, n: int, snps, missing_q24: int = 0, samples=None) -> np.ndarray:
    """Genotype codes (samples x SNPs, uint8; 3 = missing) of the generator.

    Same arithmetic as the device generator: one 64-bit hash per
    (SNP, sample); two Bernoulli(MAF) alleles from bits 0-23 and 24-47,
    missing if bits 48-63 * 256 < missing_q24.
    """
    s = np.asarray(snps, dtype=np.uint64).reshape(-1)
    i = (np.arange(n, dtype=np.uint64) if samples is None
         else np.asarray(samples, dtype=np.uint64).reshape(-1))
    with np.errstate(over="ignore"):
        key_s = _splitmix64(np.full(s.shape, seed, dtype=np.uint64) ^ (s * _U(0x8CB92BA72F3D8DD7)))
        key = key_s[None, :] ^ (i[:, None] * _U(0x9E3779B97F4A7C15))
    h = _splitmix64(key)
    maf = synth_maf_q24(seed, s).astype(np.uint64)[None, :]
    a1 = (h & _U(0xFFFFFF)) < maf
    a2 = ((h >> _U(24)) & _U(0xFFFFFF)) < maf
    codes = a1.astype(np.uint8) + a2.astype(np.uint8)
    if missing_q24:
        miss = ((h >> _U(48)) * _U(256)) < _U(missing_q24)
        codes[miss] = MISSING
    return codes


# ------------------------------------------------------------- packed format

def call_geometry(m: int, call_width: int, component_sizes=None):
    """Call blocks of width <= call_width inside each component.

    Returns (starts, widths, component_ids, component_call_offsets) as in
    geno_stream.py:469-505.
    """
    sizes = [int(m)] if component_sizes is None else [int(x) for x in component_sizes]
    if sum(sizes) != int(m):
        raise ValueError("component sizes must sum to m")
    starts, widths, comps, offsets = [], [], [], [0]
    pos = 0
    for g, size in enumerate(sizes):
        left = size
        while left > 0:
            w = min(int(call_width), left)
            starts.append(pos)
            widths.append(w)
            comps.append(g)
            pos += w
            left -= w
        offsets.append(len(starts))
    return (np.asarray(starts, np.int64), np.asarray(widths, np.int32),
            np.asarray(comps, np.int32), np.asarray(offsets, np.int32))


def codes_from_int8(block: np.ndarray, missing_val: int) -> np.ndarray:
    """Source int8 genotypes -> packed codes: 1->1, 2->2, missing->3, else 0.

    (geno_stream.py:1258-1264)
    """
    raw = np.asarray(block).view(np.uint8) if np.asarray(block).dtype == np.int8 else np.asarray(block)
    lut = np.zeros(256, dtype=np.uint8)
    lut[1] = 1
    lut[2] = 2
    lut[int(np.asarray([missing_val], dtype=np.int8).view(np.uint8)[0])] = MISSING
    return lut[raw.astype(np.uint8)]


def pack_block(codes: np.ndarray) -> np.ndarray:
    """(n, w) codes -> (n, ceil(w/4)) bytes; SNP 4j+s at bits 2s of byte j."""
    n, w = codes.shape
    pw = (w + 3) // 4
    padded = np.zeros((n, 4 * pw), dtype=np.uint8)
    padded[:, :w] = codes
    q = padded.reshape(n, pw, 4)
    return (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)


def unpack_block(packed: np.ndarray, width: int | None = None) -> np.ndarray:
    """Inverse of pack_block (kv_impl.py:58-66)."""
    p = np.asarray(packed, dtype=np.uint8)
    out = np.stack([(p >> s) & 3 for s in (0, 2, 4, 6)], axis=2).reshape(p.shape[0], -1)
    return out if width is None else out[:, :width]


def pack_calls(codes: np.ndarray, widths) -> np.ndarray:
    """Concatenate the packed call blocks of a (n, m) code matrix."""
    parts, pos = [], 0
    for w in widths:
        parts.append(pack_block(codes[:, pos:pos + int(w)]).reshape(-1))
        pos += int(w)
    return np.concatenate(parts) if parts else np.zeros(0, np.uint8)


# ------------------------------------------------------------------- stats

def raw_counts(codes: np.ndarray, sample_mask=None):
    """Per-SNP observed count, allele sum and squared allele sum."""
    c = np.asarray(codes)
    if sample_mask is not None:
        c = c[np.asarray(sample_mask, dtype=bool)]
    obs = c != MISSING
    v = np.where(obs, c, 0).astype(np.int64)
    return obs.sum(axis=0).astype(np.int64), v.sum(axis=0), (v * v).sum(axis=0)


def fp32_stats(cnt, s1, s2):
    """FP32 mean / inverse sd exactly as the reference evaluates them.

    Every step is a separately rounded float32 operation
    (geno_stream.py:1780-1792).
    """
    cnt_f = np.asarray(cnt).astype(np.float32)
    s1_f = np.asarray(s1).astype(np.float32)
    s2_f = np.asarray(s2).astype(np.float32)
    denom = np.maximum(cnt_f, np.float32(1.0))
    mean = (s1_f / denom).astype(np.float32)
    second = (s2_f / denom).astype(np.float32)
    var = np.maximum((second - (mean * mean).astype(np.float32)).astype(np.float32), np.float32(0.0))
    valid = (cnt_f > 0.0) & (var > 0.0)
    sd = np.sqrt(np.maximum(var, np.float32(1e-6))).astype(np.float32)
    inv = np.where(valid, (np.float32(1.0) / sd).astype(np.float32), np.float32(0.0)).astype(np.float32)
    return mean, inv


def stats(codes: np.ndarray, sample_mask=None):
    cnt, s1, s2 = raw_counts(codes, sample_mask)
    mean, inv = fp32_stats(cnt, s1, s2)
    return mean, inv, cnt


def stats_summary(cnt, s1, s2, mean, inv, n_sub, component_sizes=None, override=False):
    """Per-component m_eff and mean-diagonal atoms (geno_stream.py:1409-1444)."""
    sizes = [len(mean)] if component_sizes is None else list(component_sizes)
    valid = np.asarray(inv) > 0
    if override:
        mass = np.maximum(
            np.asarray(s2, np.float64) - 2.0 * np.asarray(mean, np.float64) * np.asarray(s1, np.float64)
            + np.asarray(cnt, np.float64) * np.asarray(mean, np.float64) ** 2, 0.0,
        ) * np.asarray(inv, np.float64) ** 2
    else:
        mass = np.asarray(cnt, np.float64)
    effs, atoms, pos = [], [], 0
    for size in sizes:
        sl = slice(pos, pos + int(size))
        eff = float(np.count_nonzero(valid[sl]))
        effs.append(eff)
        atoms.append(float(np.sum(mass[sl][valid[sl]]) / (n_sub * eff)) if eff > 0 else 0.0)
        pos += int(size)
    eff_total = float(np.count_nonzero(valid))
    atom_total = float(np.sum(mass[valid]) / (n_sub * eff_total)) if eff_total > 0 else 0.0
    return np.asarray(effs), np.asarray(atoms), eff_total, atom_total


# ---------------------------------------------------------------- operator

def diff_f64(codes: np.ndarray, mean, sample_mask=None) -> np.ndarray:
    """Mean-imputed, centred genotypes in FP64 (kv_impl.py:69-91)."""
    c = np.asarray(codes)
    d = c.astype(np.float64) - np.asarray(mean, np.float64)[None, :]
    d[c == MISSING] = 0.0
    if sample_mask is not None:
        d[~np.asarray(sample_mask, dtype=bool)] = 0.0
    return d


def _blocks(m: int, width: int = 4096):
    for s0 in range(0, m, width):
        yield slice(s0, min(m, s0 + width))


def kv_f64(codes, mean, inv, V, *, comp_of_snp=None, comp_scale=None, sample_mask=None,
           stacked=False, n_components=1, theta_e=None, snp_weight=None):
    """sum_g scale_g Z_g Z_g^T V (+ theta_e V) or the stacked per-component form."""
    V = np.asarray(V, np.float64)
    vec = V.ndim == 1
    if vec:
        V = V[:, None]
    n, m = np.asarray(codes).shape
    comp = np.zeros(m, np.int64) if comp_of_snp is None else np.asarray(comp_of_snp, np.int64)
    scale = np.ones(n_components) if comp_scale is None else np.asarray(comp_scale, np.float64)
    w = np.asarray(inv, np.float64) ** 2 * scale[comp]
    if snp_weight is not None:
        w = w * np.asarray(snp_weight, np.float64)
    mask = None if sample_mask is None else np.asarray(sample_mask, bool)
    Vm = V if mask is None else V * mask[:, None]
    G = n_components if stacked else 1
    out = np.zeros((G, n, V.shape[1]))
    for sl in _blocks(m):
        d = diff_f64(codes[:, sl], mean[sl], mask)
        S = w[sl, None] * (d.T @ Vm)
        if stacked:
            for g in range(G):
                sel = comp[sl] == g
                if np.any(sel):
                    out[g] += d[:, sel] @ S[sel]
        else:
            out[0] += d @ S
    if not stacked:
        out = out[0]
        if theta_e is not None:
            out = out + float(theta_e) * Vm
        return out[:, 0] if vec else out
    return out[:, :, 0] if vec else out


def xtv_f64(codes, mean, inv, V, *, scale=1.0, sample_mask=None):
    """inv_sd * (diff^T V) (kv_impl.py:163-185)."""
    V = np.asarray(V, np.float64)
    vec = V.ndim == 1
    if vec:
        V = V[:, None]
    mask = None if sample_mask is None else np.asarray(sample_mask, bool)
    Vm = V if mask is None else V * mask[:, None]
    m = np.asarray(codes).shape[1]
    out = np.zeros((m, V.shape[1]))
    for sl in _blocks(m):
        d = diff_f64(codes[:, sl], mean[sl], mask)
        out[sl] = (np.asarray(inv[sl], np.float64) * scale)[:, None] * (d.T @ Vm)
    return out[:, 0] if vec else out


def zxb_f64(codes, mean, inv, b, sample_mask=None):
    """sum_j diff_ij inv_j b_j (kv_impl.py:221-265)."""
    b = np.asarray(b, np.float64)
    vec = b.ndim == 1
    if vec:
        b = b[:, None]
    mask = None if sample_mask is None else np.asarray(sample_mask, bool)
    n, m = np.asarray(codes).shape
    out = np.zeros((n, b.shape[1]))
    for sl in _blocks(m):
        d = diff_f64(codes[:, sl], mean[sl], mask)
        out += d @ (np.asarray(inv[sl], np.float64)[:, None] * b[sl])
    return out[:, 0] if vec else out


def exact_diag(codes, mean, inv, eff, sample_mask=None):
    """diag(K)_i = sum_j z_ij^2 / m_eff in FP64 (geno_stream.py:929-955)."""
    n, m = np.asarray(codes).shape
    tot = np.zeros(n)
    mask = None if sample_mask is None else np.asarray(sample_mask, bool)
    for sl in _blocks(m):
        z = diff_f64(codes[:, sl], mean[sl], mask) * np.asarray(inv[sl], np.float64)[None, :]
        tot += np.sum(z * z, axis=1)
    return (tot / eff if eff > 0 else tot).astype(np.float32)


def kv_streamed_fp32(packed_calls: list, widths, means_by_call, inv_by_call, eff_m, V,
                     normalize=True):
    """FP32 restatement of kv_impl_streamed (kv_impl.py:94-113, :268-326).

    Per call block: unpack to uint8, impute missing with the mean, centre,
    ``inner = diff^T V``, ``acc += diff @ (inv^2 * inner)``; then divide by
    m_eff.  The two contractions use numpy's FP32 BLAS.
    """
    V = np.asarray(V, np.float32)
    vec = V.ndim == 1
    if vec:
        V = V[:, None]
    acc = np.zeros((V.shape[0], V.shape[1]), np.float32)
    for c, (blk, w) in enumerate(zip(packed_calls, widths)):
        g = unpack_block(blk)
        width = g.shape[1]
        mean_s = np.asarray(means_by_call[c][:width], np.float32)
        inv_s = np.asarray(inv_by_call[c][:width], np.float32)
        cmask = (np.arange(width) < int(w)).astype(np.float32)
        inv_f = inv_s * cmask
        g_f = g.astype(np.float32)
        g_imp = np.where(g == MISSING, mean_s[None, :], g_f)
        diff = g_imp - mean_s[None, :]
        inner = diff.T @ V
        acc += diff @ ((inv_f * inv_f)[:, None] * inner)
    if normalize and eff_m > 0:
        acc = acc / np.float32(eff_m)
    return acc[:, 0] if vec else acc


def projected_core_atom_f64(codes, mean, inv, U, eff, subtract_identity=True):
    """(Z^T U)^T (Z^T U) / m_eff (- I) (kv_impl.py:188-218, :1190-1229)."""
    XtU = xtv_f64(codes, mean, inv, U)
    core = XtU.T @ XtU
    if eff > 0:
        core = core / eff
        if subtract_identity:
            core = core - np.eye(core.shape[0])
    else:
        core = np.zeros_like(core)
    return core
