"""CPU checks of the genotype oracle: format, statistics, operator identities."""
import numpy as np
import pytest

from oracle import geno as og
from coherit_gb300 import synth


def test_generator_matches_product_generator():
    snps = np.arange(0, 300, 7)
    a = og.synth_codes(11, 50, snps, missing_q24=synth.missing_rate_q24(0.05))
    b = synth.genotype_codes(11, 50, snps, missing_q24=synth.missing_rate_q24(0.05))
    np.testing.assert_array_equal(a, b)
    assert set(np.unique(a)) <= {0, 1, 2, 3}
    assert 0.02 < np.mean(a == 3) < 0.08


def test_generator_maf_distribution():
    maf = og.synth_maf_q24(3, np.arange(20000)) / float(1 << 24)
    assert maf.min() >= 0.05 and maf.max() < 0.5
    assert abs(maf.mean() - 0.275) < 0.01
    codes = og.synth_codes(3, 4000, np.arange(200))
    freq = codes.mean(axis=0) / 2
    expect = og.synth_maf_q24(3, np.arange(200)) / float(1 << 24)
    assert np.max(np.abs(freq - expect)) < 0.05


def test_pack_unpack_round_trip_and_bit_positions():
    rng = np.random.default_rng(0)
    codes = rng.integers(0, 4, size=(5, 13)).astype(np.uint8)
    packed = og.pack_block(codes)
    assert packed.shape == (5, 4)
    # SNP 4j+s at bits 2s of byte j
    assert ((packed[:, 1] >> 4) & 3 == codes[:, 6]).all()
    np.testing.assert_array_equal(og.unpack_block(packed, 13), codes)


def test_int8_lut_matches_reference_convention():
    blk = np.asarray([[0, 1, 2, -127, 5]], dtype=np.int8)
    np.testing.assert_array_equal(og.codes_from_int8(blk, -127), [[0, 1, 2, 3, 0]])


def test_call_geometry_partitions_components():
    starts, widths, comps, offs = og.call_geometry(10, 4, [7, 3])
    assert widths.tolist() == [4, 3, 3]
    assert starts.tolist() == [0, 4, 7]
    assert comps.tolist() == [0, 0, 1]
    assert offs.tolist() == [0, 2, 3]


def test_fp32_stats_follow_float32_rounding():
    codes = og.synth_codes(5, 333, np.arange(64), missing_q24=synth.missing_rate_q24(0.1))
    mean, inv, cnt = og.stats(codes)
    c = codes.astype(np.float64)
    obs = codes != 3
    mu64 = np.where(obs, c, 0).sum(0) / obs.sum(0)
    assert np.max(np.abs(mean - mu64)) < 1e-6
    var64 = np.where(obs, (c - mu64) ** 2, 0).sum(0) / obs.sum(0)
    np.testing.assert_allclose(inv, 1 / np.sqrt(var64), rtol=1e-4)
    assert mean.dtype == np.float32 and inv.dtype == np.float32
    # monomorphic SNP -> inv_sd 0
    mono = np.zeros((10, 1), np.uint8)
    _, inv0, _ = og.stats(mono)
    assert inv0[0] == 0


def test_operator_equals_dense_grm():
    rng = np.random.default_rng(1)
    codes = og.synth_codes(2, 120, np.arange(300), missing_q24=synth.missing_rate_q24(0.03))
    mean, inv, cnt = og.stats(codes)
    eff = float(np.count_nonzero(inv > 0))
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)[None, :]
    K = Z @ Z.T / eff
    V = rng.normal(size=(120, 5))
    out = og.kv_f64(codes, mean, inv, V, comp_scale=[1 / eff])
    np.testing.assert_allclose(out, K @ V, rtol=1e-9, atol=1e-9)
    # stacked / weighted forms
    comp = np.repeat([0, 1], [100, 200])
    st = og.kv_f64(codes, mean, inv, V, comp_of_snp=comp, comp_scale=[2.0, 3.0], stacked=True,
                   n_components=2)
    Z0, Z1 = Z[:, :100], Z[:, 100:]
    np.testing.assert_allclose(st[0], 2 * Z0 @ (Z0.T @ V), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(st[1], 3 * Z1 @ (Z1.T @ V), rtol=1e-9, atol=1e-9)
    wsum = og.kv_f64(codes, mean, inv, V, comp_of_snp=comp, comp_scale=[2.0, 3.0],
                     n_components=2, theta_e=0.5)
    np.testing.assert_allclose(wsum, st[0] + st[1] + 0.5 * V, rtol=1e-9, atol=1e-9)
    # X^T V and Z b
    np.testing.assert_allclose(og.xtv_f64(codes, mean, inv, V), Z.T @ V, rtol=1e-9, atol=1e-9)
    b = rng.normal(size=(300, 2))
    np.testing.assert_allclose(og.zxb_f64(codes, mean, inv, b), Z @ b, rtol=1e-9, atol=1e-9)
    d = og.exact_diag(codes, mean, inv, eff)
    np.testing.assert_allclose(d, np.diag(K), rtol=1e-6)


def test_streamed_fp32_port_matches_fp64():
    rng = np.random.default_rng(2)
    n, m, W = 200, 700, 256
    codes = og.synth_codes(4, n, np.arange(m), missing_q24=synth.missing_rate_q24(0.02))
    mean, inv, _ = og.stats(codes)
    eff = float(np.count_nonzero(inv > 0))
    starts, widths, _, _ = og.call_geometry(m, W)
    blocks = [og.pack_block(codes[:, s:s + w]) for s, w in zip(starts, widths)]
    mbc = np.zeros((len(widths), 4 * ((W + 3) // 4)), np.float32)
    ibc = np.zeros_like(mbc)
    for c, (s, w) in enumerate(zip(starts, widths)):
        mbc[c, :w] = mean[s:s + w]
        ibc[c, :w] = inv[s:s + w]
    V = rng.normal(size=(n, 3)).astype(np.float32)
    out32 = og.kv_streamed_fp32(blocks, widths, mbc, ibc, eff, V)
    out64 = og.kv_f64(codes, mean, inv, V, comp_scale=[1 / eff])
    np.testing.assert_allclose(out32, out64, rtol=2e-5, atol=2e-5)


def test_subset_mask_operator():
    rng = np.random.default_rng(3)
    codes = og.synth_codes(8, 90, np.arange(150))
    mask = rng.random(90) < 0.6
    mean, inv, cnt = og.stats(codes, mask)
    sub = codes[mask]
    mean_s, inv_s, _ = og.stats(sub)
    np.testing.assert_array_equal(mean, mean_s)
    V = rng.normal(size=(90, 2))
    out = og.kv_f64(codes, mean, inv, V, sample_mask=mask)
    ref = og.kv_f64(sub, mean_s, inv_s, V[mask])
    np.testing.assert_allclose(out[mask], ref, rtol=1e-9, atol=1e-9)
    assert np.all(out[~mask] == 0)


@pytest.mark.parametrize("override", [False, True])
def test_stats_summary_atoms(override):
    codes = og.synth_codes(9, 50, np.arange(40), missing_q24=synth.missing_rate_q24(0.1))
    cnt, s1, s2 = og.raw_counts(codes)
    mean, inv = og.fp32_stats(cnt, s1, s2)
    effs, atoms, et, at = og.stats_summary(cnt, s1, s2, mean, inv, 50, [25, 15], override=override)
    assert effs.sum() == et
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)
    if override:
        np.testing.assert_allclose(at, np.sum(Z * Z) / (50 * et), rtol=1e-9, atol=1e-9)
    else:
        np.testing.assert_allclose(at, np.sum(cnt[inv > 0]) / (50 * et), rtol=1e-9, atol=1e-9)
