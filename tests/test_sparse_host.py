"""Host-side checks of the rare-variant path that need no GPU: shard
argument validation of the kv_impl shims, the sparse C ABI's validation of
host entry lists (both reject before touching a device), the entry lists a
host source yields, and the synthetic rare-variant source, against the
oracle."""
import ctypes as C

import numpy as np
import pytest

from coherit_gb300 import _lib, kv_impl


def test_shard_arrays_must_agree():
    with pytest.raises(ValueError, match="one length"):
        kv_impl._TransientSparse(10, 3, np.zeros(3), np.ones(3), [0, 1], [0], [1], None)
    with pytest.raises(ValueError, match="ascending"):
        kv_impl._TransientSparse(10, 3, np.zeros(3), np.ones(3), [0, 1], [2, 1],
                                 np.asarray([1, 1], np.int8), None)
    with pytest.raises(ValueError, match="ascending"):
        kv_impl._TransientSparse(10, 3, np.zeros(3), np.ones(3), [0], [3],
                                 np.asarray([1], np.int8), None)
    with pytest.raises(ValueError, match="m=3"):
        kv_impl._TransientSparse(10, 3, np.zeros(2), np.ones(3), [0], [0],
                                 np.asarray([1], np.int8), None)


@pytest.mark.parametrize("case,status", [
    ("offset0", _lib.E_SHAPE),
    ("decreasing", _lib.E_SHAPE),
    ("row", _lib.E_INDEX),
    ("value", _lib.E_SHAPE),
])
def test_csc_entry_lists_validated_before_device_use(case, status):
    lib = _lib.load()
    col_off = np.asarray([0, 2, 3], np.int64)
    rows = np.asarray([0, 4, 2], np.int32)
    vals = np.asarray([1, 2, 3], np.int8)
    if case == "offset0":
        col_off = np.asarray([1, 2, 3], np.int64)
    elif case == "decreasing":
        col_off = np.asarray([0, 3, 2], np.int64)
    elif case == "row":
        rows = np.asarray([0, 9, 2], np.int32)
    elif case == "value":
        vals = np.asarray([1, 0, 3], np.int8)
    h = C.c_void_p()
    rc = lib.coherit_sparse_create_csc(5, 2, col_off.ctypes.data, rows.ctypes.data,
                                       vals.ctypes.data, 0, None, C.byref(h))
    assert rc == status
    assert not h
    assert _lib.last_error()


def test_null_sparse_handle_is_rejected():
    lib = _lib.load()
    assert lib.coherit_sparse_info(None, None, None, None, None, None) == _lib.E_CLOSED
    assert lib.coherit_sparse_kv(None, None, 1, 1, 1.0, 0.0, None, 1, None) == _lib.E_CLOSED


@pytest.mark.parametrize("masked", [False, True])
def test_host_entry_lists_equal_oracle(masked):
    """Per-SNP entry lists from a host source (sparse_stream.py:336-469 of the
    reference): SNP-major, samples ascending, 1 het / 2 hom-alt / 3 missing."""
    import types

    from coherit_gb300 import geno_stream as gs
    from coherit_gb300 import sparse_stream as ss
    from oracle import sparse12 as osp

    rng = np.random.default_rng(4)
    n, m = 37, 23
    g = (rng.random((n, m)) < 0.08).astype(np.int8) + (rng.random((n, m)) < 0.03).astype(np.int8)
    g[rng.random((n, m)) < 0.02] = -127
    mask = rng.random(n) < 0.7 if masked else None
    starts, widths, _, _ = gs._build_call_geometry(m, 8, [m])
    fake = types.SimpleNamespace(_n_calls=int(starts.size), _call_snp_starts=starts,
                                 _call_true_widths=widths, _sample_mask=mask, m=m)
    col_off, rows, vals = ss.SparseGenoBlockStreamer._entries_from_source(fake, gs.ArraySource(g))
    sel = g if mask is None else g[mask]
    codes = np.where(sel == -127, 3, sel).astype(np.uint8)
    ref = osp.csc_from_codes(codes)
    for got, want in zip((col_off, rows, vals), ref):
        np.testing.assert_array_equal(got, want)


def test_synthetic_rare_source_equals_oracle_generator():
    from coherit_gb300 import synth
    from coherit_gb300.sparse_stream import SyntheticRareSource
    from oracle import sparse12 as osp

    src = SyntheticRareSource(60, 40, seed=12, maf_range=(0.001, 0.04), missing_rate=0.01)
    blk = src.read_block_variant_major(5, 30)
    lo, hi = synth.maf_range_q24(0.001, 0.04)
    ref = osp.synth_rare_codes(12, 60, np.arange(5, 35), lo, hi,
                               missing_q24=synth.missing_rate_q24(0.01))
    got = np.where(blk.T == src.missing_val, 3, blk.T).astype(np.uint8)
    np.testing.assert_array_equal(got, ref)
