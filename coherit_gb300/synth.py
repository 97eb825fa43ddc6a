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

def ld_block_genotypes(seed: int, n: int, m: int, *, block: int = 200, rho_range=(0.0, 0.9),
                       maf_range=(0.05, 0.5)):
    """Genotypes with linkage disequilibrium inside blocks of ``block`` SNPs.

    Each block draws rho ~ U(rho_range); every sample carries two latent
    haplotype chains h_0 ~ N(0, 1), h_j = rho h_{j-1} + sqrt(1 - rho^2) e_j,
    and allele j is 1[h_j < Phi^-1(p_j)] with p_j ~ U(maf_range).  Each allele
    is Bernoulli(p_j), so genotypes (two alleles) are in Hardy-Weinberg
    equilibrium, and neighbouring SNPs are correlated through rho; blocks are
    independent.  Host-side, for test-sized matrices.

    Returns (codes (n, m) uint8 in {0, 1, 2}, maf (m,), rho per block).
    """
    from scipy.stats import norm

    if block < 1:
        raise ValueError("block must be positive")
    lo, hi = (float(x) for x in rho_range)
    if not 0.0 <= lo <= hi < 1.0:
        raise ValueError("rho_range must satisfy 0 <= lo <= hi < 1")
    rng = np.random.default_rng(seed)
    maf = rng.uniform(maf_range[0], maf_range[1], size=m)
    thr = norm.ppf(maf)
    n_blocks = (m + block - 1) // block
    rho = rng.uniform(lo, hi, size=n_blocks)
    codes = np.zeros((n, m), dtype=np.uint8)
    for b in range(n_blocks):
        j0, j1 = b * block, min((b + 1) * block, m)
        r, s = rho[b], np.sqrt(1.0 - rho[b] ** 2)
        h = rng.normal(size=(2, n))
        for j in range(j0, j1):
            if j > j0:
                h = r * h + s * rng.normal(size=(2, n))
            codes[:, j] = (h[0] < thr[j]).astype(np.uint8) + (h[1] < thr[j]).astype(np.uint8)
    return codes, maf, rho


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
