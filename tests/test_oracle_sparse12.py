"""Pins of the rare-variant sparse oracle (CPU).

The reference has no tests or golden vectors for its sparse path, so its
restatement is pinned against the dense FP64 oracle on the same genotype
codes: the shard decomposition row_sparse + row_b sum_v + base
(kv_impl.py:777-817) must equal Z Z^T V / m_eff to rounding, X^T V and the
projected-core atom likewise, and the single-pass BED build must reproduce
the dense statistics bit for bit.  Edge columns: no entries, all missing,
monomorphic het (zero variance), and a sample subset."""
import numpy as np
import pytest

from coherit_gb300 import synth
from coherit_gb300.bed import write_bed
from oracle import geno as og
from oracle import sparse12 as osp


def _codes(seed=3, n=300, m=120, missing=0.02):
    codes = osp.rare_codes(seed, n, m, maf_lo=0.002, maf_hi=0.05, missing=missing)
    codes[:, 0] = 0           # no entries
    codes[:, 1] = osp.MISS    # all missing
    codes[:, 2] = 1           # monomorphic het: zero variance
    codes[::7, 3] = 2         # a hom-alt only column
    return codes


def _rel(a, b):
    return np.max(np.linalg.norm(a - b, axis=0) / np.maximum(np.linalg.norm(b, axis=0), 1e-300))


def test_entry_lists_order_and_values():
    codes = _codes()
    col_off, rows, vals = osp.csc_from_codes(codes)
    assert col_off[0] == 0 and col_off[-1] == rows.size == np.count_nonzero(codes)
    assert col_off[1] - col_off[0] == 0
    for j in range(codes.shape[1]):
        r = rows[col_off[j]:col_off[j + 1]]
        assert np.all(np.diff(r) > 0)
        np.testing.assert_array_equal(r, np.flatnonzero(codes[:, j]))
        np.testing.assert_array_equal(vals[col_off[j]:col_off[j + 1]], codes[r, j])


def test_stats_equal_dense_oracle():
    codes = _codes()
    st = osp.bed_counts_stats(codes)
    mean, inv, cnt = og.stats(codes)
    np.testing.assert_array_equal(st["mean"], mean)
    np.testing.assert_array_equal(st["inv"], inv)
    np.testing.assert_array_equal(st["cnt"], cnt)
    assert inv[0] == 0 and inv[1] == 0 and inv[2] == 0
    _, s1, s2 = og.raw_counts(codes)
    _, _, eff, atom = og.stats_summary(cnt, s1, s2, mean, inv, codes.shape[0])
    assert st["eff"] == eff
    assert st["atom"] == pytest.approx(atom, rel=1e-15)


@pytest.mark.parametrize("k", [1, 4, 7])
def test_shard_decomposition_equals_dense_operator(k):
    codes = _codes(seed=5 + k)
    mean, inv, _ = og.stats(codes)
    eff = float(np.count_nonzero(inv > 0))
    csc = osp.csc_from_codes(codes)
    V = np.random.default_rng(k).normal(size=(codes.shape[0], k)) + 0.3
    got = osp.kv_f64(*csc, mean, inv, V, eff)
    ref = og.kv_f64(codes, mean, inv, V, comp_scale=[1.0 / eff])
    assert _rel(got, ref) < 1e-12
    np.testing.assert_allclose(osp.xtv_f64(*csc, mean, inv, V), og.xtv_f64(codes, mean, inv, V),
                               rtol=1e-11, atol=1e-11)
    core = osp.projected_core_atom_f64(*csc, mean, inv, V, eff)
    np.testing.assert_allclose(core, og.projected_core_atom_f64(codes, mean, inv, V, eff),
                               rtol=1e-10, atol=1e-10)


def test_vector_right_hand_side():
    codes = _codes(seed=11)
    mean, inv, _ = og.stats(codes)
    csc = osp.csc_from_codes(codes)
    v = np.random.default_rng(0).normal(size=codes.shape[0])
    a = osp.kv_f64(*csc, mean, inv, v, 10.0)
    b = osp.kv_f64(*csc, mean, inv, v[:, None], 10.0)[:, 0]
    np.testing.assert_array_equal(a, b)


def test_bed_decode_round_trip_and_keep_list(tmp_path):
    codes = _codes(seed=13, n=203, m=37)
    prefix = str(tmp_path / "r")
    write_bed(prefix, np.where(codes == 3, -1, codes.astype(np.int16)))
    raw = np.fromfile(prefix + ".bed", dtype=np.uint8)
    np.testing.assert_array_equal(osp.codes_from_bed(raw, 203, 37), codes)
    keep = np.flatnonzero(np.random.default_rng(1).random(203) < 0.5)
    np.testing.assert_array_equal(osp.codes_from_bed(raw, 203, 37, keep), codes[keep])
    with pytest.raises(ValueError):
        osp.codes_from_bed(raw[1:], 203, 37)


def test_all_invalid_snps_give_zero_operator():
    codes = np.zeros((50, 4), dtype=np.uint8)
    codes[:, 1] = osp.MISS
    mean, inv, _ = og.stats(codes)
    csc = osp.csc_from_codes(codes)
    V = np.ones((50, 2))
    np.testing.assert_array_equal(osp.kv_f64(*csc, mean, inv, V, 0.0), np.zeros((50, 2)))
    assert osp.projected_core_atom_f64(*csc, mean, inv, V, 0.0).tolist() == [[0, 0], [0, 0]]


def test_rare_generator_restatement():
    """The rare-variant generator is the dense generator with another MAF
    range: with the dense range it reproduces the dense oracle exactly, and
    the product's host evaluation equals the oracle's for a rare range."""
    snps = np.arange(40)
    lo, hi = synth.COMMON_MAF_Q24
    np.testing.assert_array_equal(osp.synth_rare_codes(9, 500, snps, lo, hi, 4096),
                                  og.synth_codes(9, 500, snps, missing_q24=4096))
    r = synth.maf_range_q24(0.0005, 0.01)
    codes = osp.synth_rare_codes(9, 500, snps, *r, missing_q24=4096)
    np.testing.assert_array_equal(synth.genotype_codes(9, 500, snps, 4096, r), codes)
    maf = osp.synth_maf_q24_range(9, snps, *r) / float(1 << 24)
    assert np.all((maf >= 0.0005 - 1e-9) & (maf < 0.01))
    with pytest.raises(ValueError):
        synth.maf_range_q24(0.2, 0.1)
