"""Synthetic genotypes and phenotypes of the benchmark configurations.

Genotypes come from a counter-based hash of (seed, SNP, sample): per-SNP MAF
~ U(0.05, 0.5) and two Bernoulli(MAF) alleles (Hardy-Weinberg), optionally a
missing code.  The CUDA library evaluates the same hash on the device to
write the resident matrix directly; this module evaluates it on the host for
the few SNPs a phenotype needs (its causal set).
"""
from __future__ import annotations

import numpy as np

_U = np.uint64


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x + _U(0x9E3779B97F4A7C15)
        x = (x ^ (x >> _U(30))) * _U(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> _U(27))) * _U(0x94D049BB133111EB)
    return x ^ (x >> _U(31))


COMMON_MAF_Q24 = (838861, 838861 + 7549747)  # [0.05, 0.5)


def maf_q24(seed: int, snps, maf_range_q24=COMMON_MAF_Q24) -> np.ndarray:
    """Per-SNP MAF on a 2^24 scale, uniform on [lo, hi) of ``maf_range_q24``."""
    lo, hi = (int(x) for x in maf_range_q24)
    s = np.asarray(snps, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = _splitmix64(np.full(s.shape, seed, dtype=np.uint64) * _U(0xD1B54A32D192ED03) + s)
    return (_U(lo) + (h >> _U(20)) % _U(hi - lo)).astype(np.uint32)


def maf_range_q24(lo: float, hi: float) -> tuple:
    """MAF interval [lo, hi) on the generator's 2^24 scale."""
    if not 0.0 <= lo < hi <= 0.5:
        raise ValueError("MAF range must satisfy 0 <= lo < hi <= 0.5")
    return int(round(lo * (1 << 24))), int(round(hi * (1 << 24)))


def genotype_codes(seed: int, n: int, snps, missing_q24: int = 0,
                   maf_range_q24=COMMON_MAF_Q24) -> np.ndarray:
    """Codes (n x len(snps), uint8; 3 = missing) of the given SNP indices."""
    s = np.asarray(snps, dtype=np.uint64).reshape(-1)
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key_s = _splitmix64(np.full(s.shape, seed, dtype=np.uint64) ^ (s * _U(0x8CB92BA72F3D8DD7)))
        key = key_s[None, :] ^ (i[:, None] * _U(0x9E3779B97F4A7C15))
    h = _splitmix64(key)
    maf = maf_q24(seed, s, maf_range_q24).astype(np.uint64)[None, :]
    codes = ((h & _U(0xFFFFFF)) < maf).astype(np.uint8) + (
        ((h >> _U(24)) & _U(0xFFFFFF)) < maf
    ).astype(np.uint8)
    if missing_q24:
        codes[((h >> _U(48)) * _U(256)) < _U(missing_q24)] = 3
    return codes


def missing_rate_q24(rate: float) -> int:
    if not 0.0 <= rate < 1.0:
        raise ValueError("missing rate must lie in [0, 1)")
    return int(round(rate * (1 << 24)))


def phenotype(seed: int, n: int, m: int, *, h2: float, n_causal: int, missing_q24: int = 0,
              n_covar: int = 0, pheno_seed: int | None = None, effect="normal",
              noise_var: float | None = None):
    """Phenotype with `n_causal` standardised-genotype effects scaled to h2.

    Returns (y, X, causal_idx, beta) with X = [1, N(0,1) covariates].  The
    genetic value uses standardised causal genotypes (missing -> mean), its
    variance is rescaled to h2; the noise is N(0, 1 - h2) unless noise_var
    is given.
    """
    rng = np.random.default_rng(seed if pheno_seed is None else pheno_seed)
    causal = np.sort(rng.choice(m, size=min(n_causal, m), replace=False))
    if effect == "laplace":
        beta = rng.laplace(0.0, 0.1, size=causal.size)
    else:
        beta = rng.normal(size=causal.size)
    g = np.zeros(n)
    for s0 in range(0, causal.size, 512):
        idx = causal[s0:s0 + 512]
        codes = genotype_codes(seed, n, idx, missing_q24).astype(np.float64)
        miss = codes == 3
        codes[miss] = np.nan
        mu = np.nanmean(codes, axis=0)
        sd = np.nanstd(codes, axis=0)
        sd[sd == 0] = 1.0
        z = (codes - mu) / sd
        z[np.isnan(z)] = 0.0
        g += z @ beta[s0:s0 + 512]
    vg = np.var(g)
    if vg > 0:
        g *= np.sqrt(h2 / vg)
    ve = (1.0 - h2) if noise_var is None else noise_var
    y = g + rng.normal(scale=np.sqrt(ve), size=n)
    X = np.column_stack([np.ones(n), rng.normal(size=(n, n_covar))]) if n_covar >= 0 else None
    return y.astype(np.float32), X.astype(np.float32), causal, beta


# ------------------------------------------------- block-LD genotypes (8-GRM workload)

_Q_BITS = 12


def _snp_keys(seed: int, snps) -> np.ndarray:
    s = np.asarray(snps, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _splitmix64(np.full(s.shape, seed, dtype=np.uint64) ^ (s * _U(0x8CB92BA72F3D8DD7)))


def ld_tables(seed: int, m: int, *, block: int = 200, rho_range=(0.0, 0.9),
              maf_range_q24=COMMON_MAF_Q24):
    """Tables of the block-LD generator: per-SNP thresholds Phi^-1(maf_j) and
    the population MAF, per-block rho_b ~ U(rho_range) and s_b = sqrt(1 -
    rho_b^2), and the 4096 standard-normal quantiles Phi^-1((k + 1/2) / 4096)
    the draws come from.  Returns float32 (thr, rho, s, quantiles) and the
    float64 MAF."""
    from scipy.special import ndtri

    if block < 1:
        raise ValueError("block must be positive")
    lo, hi = (float(x) for x in rho_range)
    if not 0.0 <= lo <= hi < 1.0:
        raise ValueError("rho_range must satisfy 0 <= lo <= hi < 1")
    maf = maf_q24(seed, np.arange(m), maf_range_q24).astype(np.float64) / float(1 << 24)
    thr = ndtri(maf).astype(np.float32)
    nb = (m + block - 1) // block
    b = np.arange(nb, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = _splitmix64(np.full(b.shape, seed, dtype=np.uint64) * _U(0xA24BAED4963EE407)
                        ^ (b * _U(0x9FB21C651E98DF25)))
    u = (h >> _U(40)).astype(np.float64) / float(1 << 24)
    rho = (lo + (hi - lo) * u).astype(np.float32)
    sfac = np.sqrt(1.0 - rho.astype(np.float64) ** 2).astype(np.float32)
    quant = ndtri((np.arange(1 << _Q_BITS) + 0.5) / float(1 << _Q_BITS)).astype(np.float32)
    return thr, rho, sfac, quant, maf


def ld_block_codes(seed: int, n: int, m: int, *, block: int = 200, tables=None,
                   samples=None) -> np.ndarray:
    """Codes (n x m, uint8 in {0, 1, 2}) of the block-LD generator, with the
    arithmetic of the device generator (coherit_ldblock_records): per sample,
    haplotype a and block, x_0 = e_0 and x_p = rho_b x_{p-1} + s_b e_p in
    float32 with separately rounded products and sum, e = quantiles[top 12
    bits of splitmix64(key_j ^ (2i + a) C)], allele = [x_p < thr_j].  Host
    scale (tests and small fits)."""
    thr, rho, sfac, quant, _ = tables if tables is not None else ld_tables(seed, m, block=block)
    i = np.arange(n, dtype=np.uint64) if samples is None else np.asarray(samples, np.uint64)
    codes = np.zeros((i.size, m), dtype=np.uint8)
    keys = _snp_keys(seed, np.arange(m))
    for b in range((m + block - 1) // block):
        r, sf = np.float32(rho[b]), np.float32(sfac[b])
        x = np.zeros((2, i.size), np.float32)
        for j in range(b * block, min(m, (b + 1) * block)):
            for a in range(2):
                with np.errstate(over="ignore"):
                    hh = _splitmix64(keys[j] ^ ((_U(2) * i + _U(a)) * _U(0x9E3779B97F4A7C15)))
                e = quant[(hh >> _U(64 - _Q_BITS)).astype(np.int64)]
                if j == b * block:
                    x[a] = e
                else:
                    x[a] = np.float32(r * x[a]) + np.float32(sf * e)
            codes[:, j] = (x[0] < thr[j]).astype(np.uint8) + (x[1] < thr[j]).astype(np.uint8)
    return codes


def ld_block_genotypes(seed: int, n: int, m: int, *, block: int = 200, rho_range=(0.0, 0.9),
                       maf_range=(0.05, 0.5)):
    """Genotypes with linkage disequilibrium inside blocks of ``block`` SNPs
    (the generator the device builds the 8-component workload with).

    Each block has rho_b ~ U(rho_range); every sample carries two latent
    haplotype chains x_0 ~ N(0, 1), x_p = rho_b x_{p-1} + sqrt(1 - rho_b^2)
    e_p, and allele j is 1[x_j < Phi^-1(p_j)] with p_j ~ U(maf_range).  Each
    allele is Bernoulli(p_j), so genotypes (two alleles) are in
    Hardy-Weinberg equilibrium and neighbouring SNPs correlate through rho_b;
    blocks are independent.

    Returns (codes (n, m) uint8 in {0, 1, 2}, maf (m,), rho per block).
    """
    q24 = maf_range_q24(*maf_range)
    tables = ld_tables(seed, m, block=block, rho_range=rho_range, maf_range_q24=q24)
    codes = ld_block_codes(seed, n, m, block=block, tables=tables)
    return codes, tables[4], tables[1].astype(np.float64)


def ld_partition_device(seed: int, m: int, *, block: int = 200, n_ld: int = 4096,
                        n_maf_bins: int = 4, device=None, rho_range=(0.0, 0.9)):
    """The 4 MAF bins x 2 LD-score halves partition of the block-LD generator
    at full size, built on the device: codes of the first ``n_ld`` samples
    from coherit_ldblock_records, LD scores (sum of r^2 within each block) by
    batched FP32 Gram products, MAF = the generator's population MAF.
    Returns (groups, tables)."""
    import torch

    from . import _lib

    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    tables = ld_tables(seed, m, block=block, rho_range=rho_range)
    thr, rho, sfac, quant, maf = tables
    td = [torch.as_tensor(a, device=dev).contiguous() for a in (thr, rho, sfac, quant)]
    bps = (n_ld + 3) // 4
    rec = torch.empty((m, bps), dtype=torch.uint8, device=dev)
    _lib.check(lib.coherit_ldblock_records(n_ld, m, block, seed, *(t.data_ptr() for t in td),
                                           rec.data_ptr(), _lib.stream_ptr()), "LD-block records")
    lut = torch.tensor([2.0, 0.0, 1.0, 0.0], device=dev)  # BED 0,1,2,3 -> count (no missing)
    ld = torch.empty(m, dtype=torch.float64, device=dev)
    nb = (m + block - 1) // block
    per = max(1, (1 << 28) // (block * n_ld))
    for b0 in range(0, nb, per):
        j0, j1 = b0 * block, min(m, (b0 + per) * block)
        r = rec[j0:j1]
        g = torch.stack([lut[((r >> (2 * t)) & 3).long()] for t in range(4)], dim=2)
        g = g.reshape(j1 - j0, 4 * bps)[:, :n_ld]
        g = g - g.mean(dim=1, keepdim=True)
        sd = g.std(dim=1, unbiased=False, keepdim=True)
        g = torch.where(sd > 0, g / torch.where(sd > 0, sd, torch.ones_like(sd)), torch.zeros_like(g))
        full = (j1 - j0) // block * block
        if full:
            zb = g[:full].reshape(-1, block, n_ld)
            cor = torch.bmm(zb, zb.transpose(1, 2)) / n_ld
            ld[j0:j0 + full] = (cor * cor).sum(dim=2).reshape(-1).double()
        if full < j1 - j0:
            zt = g[full:]
            cor = zt @ zt.T / n_ld
            ld[j0 + full:j1] = (cor * cor).sum(dim=1).double()
    groups = maf_ld_partition(maf, ld.cpu().numpy(), n_maf_bins=n_maf_bins)
    return groups, tables


def block_ld_scores(codes: np.ndarray, block: int = 200) -> np.ndarray:
    """LD score of each SNP: the sum of its r^2 with the SNPs of its block
    (itself included); monomorphic SNPs score 0."""
    g = np.asarray(codes, np.float64)
    n, m = g.shape
    out = np.zeros(m)
    for j0 in range(0, m, block):
        z = g[:, j0:j0 + block]
        z = z - z.mean(axis=0)
        sd = z.std(axis=0)
        z = np.where(sd > 0, z / np.where(sd > 0, sd, 1.0), 0.0)
        r = z.T @ z / n
        out[j0:j0 + z.shape[1]] = np.sum(r * r, axis=1)
    return out


def maf_ld_partition(maf, ld_scores, n_maf_bins: int = 4) -> list:
    """Component groups: MAF quantile bins, each split at its median LD score
    into a lower and an upper half.  Returns 2 * n_maf_bins sorted SNP index
    arrays ordered (bin 0 low LD, bin 0 high LD, bin 1 low LD, ...); together
    they hold every SNP once."""
    maf = np.asarray(maf, np.float64)
    ld = np.asarray(ld_scores, np.float64)
    order = np.argsort(maf, kind="stable")
    groups = []
    for part in np.array_split(order, n_maf_bins):
        by_ld = part[np.argsort(ld[part], kind="stable")]
        half = by_ld.size // 2
        groups += [np.sort(by_ld[:half]), np.sort(by_ld[half:])]
    return groups


def dirichlet_h2(seed: int, n_components: int, total: float = 0.4) -> np.ndarray:
    """Per-component heritabilities ~ Dirichlet(1, ..., 1) scaled to ``total``."""
    return total * np.random.default_rng(seed).dirichlet(np.ones(n_components))


def partitioned_phenotype(codes: np.ndarray, groups, h2s, *, seed: int, n_causal_per: int,
                          n_covar: int = 0):
    """Phenotype whose component g explains h2s[g] of the variance through
    ``n_causal_per`` standardised causal SNPs drawn from groups[g]; the rest is
    N(0, 1 - sum h2s) noise.  Returns (y float32, X float32 = [1, N(0,1) covariates])."""
    rng = np.random.default_rng(seed)
    g = np.asarray(codes, np.float64)
    n = g.shape[0]
    y = np.zeros(n)
    for grp, h2 in zip(groups, h2s):
        idx = rng.choice(np.asarray(grp), size=min(n_causal_per, len(grp)), replace=False)
        z = g[:, idx] - g[:, idx].mean(axis=0)
        sd = z.std(axis=0)
        z = np.where(sd > 0, z / np.where(sd > 0, sd, 1.0), 0.0)
        comp = z @ rng.normal(size=idx.size)
        v = np.var(comp)
        if v > 0 and h2 > 0:
            y += comp * np.sqrt(h2 / v)
    y += rng.normal(scale=np.sqrt(max(1e-6, 1.0 - float(np.sum(h2s)))), size=n)
    X = np.column_stack([np.ones(n), rng.normal(size=(n, n_covar))])
    return y.astype(np.float32), X.astype(np.float32)
