"""The block-LD genotype generator and the MAF x LD-score partition of the
8-GRM workload (host side, CPU)."""
import numpy as np
import pytest

from coherit_gb300 import synth


def test_block_ld_genotypes_hwe_and_ld():
    codes, maf, rho = synth.ld_block_genotypes(11, 4000, 600, block=200, rho_range=(0.0, 0.9))
    assert codes.shape == (4000, 600) and codes.dtype == np.uint8 and codes.max() <= 2
    assert rho.shape == (3,) and np.all((0 <= rho) & (rho < 0.9))
    again = synth.ld_block_genotypes(11, 4000, 600, block=200)
    np.testing.assert_array_equal(codes, again[0])
    # Each allele is Bernoulli(maf): allele frequency and heterozygosity of HWE.
    p_hat = codes.mean(axis=0) / 2
    assert np.max(np.abs(p_hat - maf)) < 0.04
    het = np.mean(codes == 1, axis=0)
    assert np.max(np.abs(het - 2 * maf * (1 - maf))) < 0.05
    # Neighbours correlate through the block's rho; blocks are independent.
    g = codes.astype(np.float64)
    g = (g - g.mean(axis=0)) / g.std(axis=0)
    adj = np.array([np.mean(g[:, j] * g[:, j + 1]) for j in range(599) if (j + 1) % 200])
    per_block = adj.reshape(3, 199).mean(axis=1)
    assert np.all(np.diff(per_block[np.argsort(rho)]) > 0)
    across = [np.mean(g[:, 200 * b - 1] * g[:, 200 * b]) for b in (1, 2)]
    assert np.max(np.abs(across)) < 0.06


def test_ld_scores_follow_rho():
    codes, maf, rho = synth.ld_block_genotypes(3, 3000, 800, block=200)
    ld = synth.block_ld_scores(codes)
    assert np.all(ld >= 1.0 - 1e-9)
    means = ld.reshape(4, 200).mean(axis=1)
    assert np.argmax(means) == np.argmax(rho) and np.argmin(means) == np.argmin(rho)
    mono = np.zeros((10, 5), np.uint8)
    np.testing.assert_array_equal(synth.block_ld_scores(mono), 0.0)


def test_maf_ld_partition_is_exhaustive_and_ordered():
    rng = np.random.default_rng(0)
    maf = rng.uniform(0.05, 0.5, size=1001)
    ld = rng.uniform(1, 5, size=1001)
    groups = synth.maf_ld_partition(maf, ld)
    assert len(groups) == 8
    np.testing.assert_array_equal(np.sort(np.concatenate(groups)), np.arange(1001))
    for grp in groups:
        assert np.all(np.diff(grp) > 0)
    # Bins increase in MAF; within a bin the second half has the larger LD scores.
    for b in range(4):
        lo_ld, hi_ld = groups[2 * b], groups[2 * b + 1]
        assert ld[lo_ld].max() <= ld[hi_ld].min()
        if b:
            prev = np.concatenate(groups[2 * b - 2: 2 * b])
            cur = np.concatenate(groups[2 * b: 2 * b + 2])
            assert maf[prev].max() <= maf[cur].min()


def test_dirichlet_h2_and_partitioned_phenotype():
    h2 = synth.dirichlet_h2(5, 8, total=0.4)
    assert h2.shape == (8,) and np.all(h2 > 0) and h2.sum() == pytest.approx(0.4)
    np.testing.assert_array_equal(h2, synth.dirichlet_h2(5, 8, total=0.4))
    codes, maf, _ = synth.ld_block_genotypes(2, 3000, 400, block=100)
    groups = synth.maf_ld_partition(maf, synth.block_ld_scores(codes, block=100))
    y, X = synth.partitioned_phenotype(codes, groups, h2, seed=9, n_causal_per=10, n_covar=3)
    assert y.shape == (3000,) and X.shape == (3000, 4)
    assert np.var(y) == pytest.approx(1.0, rel=0.15)
    with pytest.raises(ValueError):
        synth.ld_block_genotypes(0, 10, 10, rho_range=(0.5, 1.0))
