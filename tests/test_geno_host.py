"""Host side of the genotype streamer on CPU: call geometry, packing, BED reading.

Everything here runs before the first device call of ``GenoBlockStreamer``:
the call blocks inside each component (geno_stream.py:469-505 of the
reference), the source -> 2-bit packed bytes conversion for sources that are
not built on the device (geno_stream.py:1258-1264, :709-745), and the PLINK
BED reader.  The product refuses to run without a CUDA device; that is
checked here too.
"""
import types

import numpy as np
import pytest
import torch

from coherit_gb300 import bed, geno_stream as gs
from oracle import geno as og
from oracle import sparse12 as osp


@pytest.mark.parametrize("m,width,sizes", [
    (10, 4, None), (131072, 131072, None), (131073, 131072, None), (17, 5, [3, 9, 5]),
    (1000, 256, [1, 999]), (12, 100, [4, 4, 4]),
])
def test_call_geometry_equals_oracle(m, width, sizes):
    got = gs._build_call_geometry(m, width, sizes or [m])
    ref = og.call_geometry(m, width, sizes)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
        assert a.dtype == b.dtype
    starts, widths, comps, offsets = got
    assert np.all(widths <= width) and widths.sum() == m
    np.testing.assert_array_equal(starts[1:], np.cumsum(widths)[:-1])


@pytest.mark.parametrize("missing_val", [-127, -1, 3, 9])
@pytest.mark.parametrize("w", [1, 3, 4, 7, 64, 129])
def test_pack_block_equals_oracle(missing_val, w):
    rng = np.random.default_rng(w)
    n = 37
    g = rng.integers(0, 3, size=(n, w)).astype(np.int8)
    g[rng.random(size=g.shape) < 0.1] = missing_val
    packed = gs._pack_block_vm(np.ascontiguousarray(g.T), gs._pack_lut(missing_val))
    ref = og.pack_block(og.codes_from_int8(g, missing_val))
    np.testing.assert_array_equal(packed, ref)
    assert packed.shape == (n, (w + 3) // 4)
    np.testing.assert_array_equal(og.unpack_block(packed, w), og.codes_from_int8(g, missing_val))


def _fake_streamer(m_source, sizes, groups=None, sample_mask=None, call_width=8):
    """The attributes ``_pack_from_source`` reads, set as the constructor sets them."""
    if groups is not None:
        sizes, cts = gs._normalize_component_variant_indices(m_source, groups)
    else:
        cts = None
    starts, widths, _, _ = gs._build_call_geometry(sum(sizes), call_width, sizes)
    st = types.SimpleNamespace(
        _cache_to_source_variant_indices=cts, _n_calls=int(starts.size),
        _call_snp_starts=starts.astype(np.int32), _call_true_widths=widths,
        _sample_mask=None if sample_mask is None else np.asarray(sample_mask, bool))
    return st, cts, widths


@pytest.mark.parametrize("case", ["whole", "blocks", "groups", "groups_masked"])
def test_pack_from_source_equals_oracle(case):
    rng = np.random.default_rng(3)
    n, m = 21, 40
    g = rng.integers(0, 3, size=(n, m)).astype(np.int8)
    g[rng.random(size=g.shape) < 0.05] = -127
    src = gs.ArraySource(g)
    mask = None
    groups = None
    sizes = [m]
    if case == "blocks":
        sizes = [7, 13, 11]
    elif case.startswith("groups"):
        perm = rng.permutation(m)
        groups = [np.sort(perm[:9]), perm[9:25], np.sort(perm[25:31])]
    if case == "groups_masked":
        mask = rng.random(n) < 0.6
    st, cts, widths = _fake_streamer(m, sizes, groups, mask)
    packed = gs.GenoBlockStreamer._pack_from_source(st, src)
    sel = g if cts is None else g[:, cts]
    sel = sel[:, : int(widths.sum())]
    if mask is not None:
        sel = sel[mask]
    ref = og.pack_calls(og.codes_from_int8(sel, -127), widths)
    np.testing.assert_array_equal(packed, ref)


def test_synthetic_source_blocks_equal_oracle_codes():
    src = gs.SyntheticSource(50, 30, seed=9, missing_rate=0.02)
    blk = src.read_block_variant_major(5, 20)
    ref = og.synth_codes(9, 50, np.arange(5, 25), missing_q24=src.missing_q24)
    np.testing.assert_array_equal(og.codes_from_int8(blk.T, src.missing_val), ref)


@pytest.mark.parametrize("n", [1, 4, 5, 33])
def test_bed_round_trip_equals_oracle_decoder(tmp_path, n):
    rng = np.random.default_rng(n)
    m = 11
    g = rng.integers(0, 3, size=(n, m)).astype(np.int8)
    g[rng.random(size=g.shape) < 0.1] = -1
    prefix = str(tmp_path / "t")
    bed.write_bed(prefix, g)
    src = bed.BedSource(prefix + ".bed")
    assert (src.n, src.m) == (n, m)
    assert src.sample_ids == tuple(f"I{i}" for i in range(n))
    got = og.codes_from_int8(src.read_block_variant_major(0, m).T, src.missing_val)
    ref = osp.codes_from_bed(np.asarray(src.raw_bytes()), n, m)
    np.testing.assert_array_equal(got, ref)
    expect = np.where(g < 0, og.MISSING, g).astype(np.uint8)
    np.testing.assert_array_equal(got, expect)
    part = og.codes_from_int8(src.read_block_variant_major(3, 5).T, src.missing_val)
    np.testing.assert_array_equal(part, expect[:, 3:8])
    src.close()


def test_bed_rejects_bad_files(tmp_path):
    g = np.zeros((6, 4), np.int8)
    prefix = str(tmp_path / "b")
    bed.write_bed(prefix, g)
    raw = open(prefix + ".bed", "rb").read()
    with open(prefix + ".bed", "wb") as f:
        f.write(raw[:-1])
    with pytest.raises(ValueError, match="does not match"):
        bed.BedSource(prefix)
    with open(prefix + ".bed", "wb") as f:
        f.write(bytes([0x6C, 0x1B, 0x00]) + raw[3:])
    with pytest.raises(ValueError, match="SNP-major"):
        bed.BedSource(prefix)


def test_array_source_contract():
    with pytest.raises(ValueError):
        gs.ArraySource(np.zeros(5))
    src = gs.ArraySource(np.arange(12, dtype=np.uint8).reshape(3, 4) % 3)
    blk = src.read_block_variant_major(1, 2)
    assert blk.dtype == np.int8 and blk.shape == (2, 3)


def test_as_rhs_shapes():
    V, squeeze = gs.as_rhs(np.arange(6.0), torch.device("cpu"))
    assert squeeze and V.shape == (6, 1) and V.dtype == torch.float32
    V, squeeze = gs.as_rhs(torch.ones((4, 3), dtype=torch.float64).T, torch.device("cpu"))
    assert not squeeze and V.is_contiguous() and V.shape == (3, 4)
    with pytest.raises(ValueError):
        gs.as_rhs(np.zeros((2, 2, 2)), torch.device("cpu"))


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_no_cpu_fallback():
    with pytest.raises(RuntimeError, match="CUDA"):
        gs._device_of(None)
    with pytest.raises(RuntimeError, match="CUDA"):
        gs.GenoBlockStreamer(gs.ArraySource(np.zeros((4, 4), np.int8)))


def test_cpu_device_is_refused():
    with pytest.raises(RuntimeError, match="CUDA devices only"):
        gs._device_of("cpu")


def test_constructor_contract_errors():
    src = gs.ArraySource(np.zeros((4, 4), np.int8))
    with pytest.raises(ValueError, match="not both"):
        gs.GenoBlockStreamer(src, bed_prefix="x")
    with pytest.raises(ValueError, match="must be provided"):
        gs.GenoBlockStreamer()


# geno_stream.py:371-437 of the reference
def test_component_variant_groups_are_sorted_into_cache_order():
    sizes, cts = gs._normalize_component_variant_indices(8, [[5, 0, 2], [4, 1, 3]])
    assert sizes == [3, 3]
    np.testing.assert_array_equal(cts, [0, 2, 5, 1, 3, 4])
    sizes, cts = gs._normalize_component_variant_indices(4, [np.array([3, 1]), [0, 2]])
    np.testing.assert_array_equal(cts, [1, 3, 0, 2])


@pytest.mark.parametrize("groups,exc,match", [
    ([], ValueError, "at least one component"),
    ([[0, 1], [1, 2]], ValueError, "disjoint"),
    ([[0, 0, 1]], ValueError, "duplicate"),
    ([[0, 4]], IndexError, "out-of-range"),
    ([[-1, 2]], IndexError, "out-of-range"),
    ([[0, 1], []], ValueError, "empty"),
])
def test_component_variant_group_errors(groups, exc, match):
    with pytest.raises(exc, match=match):
        gs._normalize_component_variant_indices(4, groups)


def test_component_block_sizes_must_cover_every_snp():
    assert gs._normalize_component_block_sizes(10, None) == [10]
    assert gs._normalize_component_block_sizes(10, np.array([3, 7])) == [3, 7]
    for sizes, match in (([], "at least one block"), ([3, 0, 7], "strictly positive"),
                         ([3, 6], "sum to m=10; got 9"), ([4, 7], "got 11")):
        with pytest.raises(ValueError, match=match):
            gs._normalize_component_block_sizes(10, sizes)
