"""PLINK BED input transcoded on the device (GPU).

The resident matrix built from a .bed file must hold exactly the genotypes
the file encodes: packed bytes read back equal the oracle's packing of the
BED codes (BED 0,1,2,3 -> 2, missing, 1, 0), FP32 statistics bit-exact, and
the operator identical to a matrix built from the same genotypes in memory.
Sample subsets (keep lists), component partitions and several transcode
chunks (SNP records spanning chunk boundaries inside one panel) included."""
import numpy as np
import pytest
import torch

from coherit_gb300 import synth
from coherit_gb300.bed import write_bed
from coherit_gb300.geno_stream import ArraySource, GenoBlockStreamer
from oracle import geno as og

pytestmark = pytest.mark.gpu


def _codes(n, m, seed, miss):
    return og.synth_codes(seed, n, np.arange(m), missing_q24=synth.missing_rate_q24(miss))


def _as_int8(codes):
    g = codes.astype(np.int8)
    g[codes == 3] = -127
    return g


@pytest.mark.parametrize("n,m,comps,mask", [
    (301, 1000, None, False),
    (257, 900, [300, 600], False),
    (400, 700, None, True),
])
def test_bed_layout_stats_and_operator(cuda, tmp_path, n, m, comps, mask):
    codes = _codes(n, m, seed=81 + n, miss=0.03)
    prefix = str(tmp_path / "g")
    write_bed(prefix, np.where(codes == 3, -1, codes.astype(np.int16)))
    keep = None
    if mask:
        keep = np.random.default_rng(2).random(n) < 0.6
    st = GenoBlockStreamer(bed_prefix=prefix, component_block_sizes=comps, call_width=256,
                           sample_mask=keep)
    sub = codes if keep is None else codes[keep]
    # Packed bytes of every call block, bit-exact.
    for c in range(st._n_calls):
        s0, w = int(st._call_snp_starts[c]), int(st._call_true_widths[c])
        np.testing.assert_array_equal(st._pop_cached(c), og.pack_block(sub[:, s0:s0 + w]))
    mean, inv, _ = og.stats(sub[:, :st.m])
    np.testing.assert_array_equal(st._means_host, mean)
    np.testing.assert_array_equal(st._inv_sds_host, inv)
    # Same operator as the in-memory build of the same genotypes.
    ref = GenoBlockStreamer(ArraySource(_as_int8(sub)), component_block_sizes=comps,
                            call_width=256)
    V = torch.randn((st.n, 5), device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    np.testing.assert_allclose(st.kv(V).cpu().numpy(), ref.kv(V).cpu().numpy(), rtol=0, atol=0)


def test_bed_chunks_split_a_panel(cuda, tmp_path, monkeypatch):
    """Small transcode chunks (97 SNP records of 1,025 bytes): 64-slot panels
    are filled by two consecutive chunks; the result equals the in-memory
    build."""
    n, m = 4099, 3000
    codes = _codes(n, m, seed=85, miss=0.01)
    prefix = str(tmp_path / "h")
    write_bed(prefix, np.where(codes == 3, -1, codes.astype(np.int16)))
    monkeypatch.setenv("COHERIT_BED_CHUNK_BYTES", str(97 * ((n + 3) // 4)))
    st = GenoBlockStreamer(bed_prefix=prefix)
    ref = GenoBlockStreamer(ArraySource(_as_int8(codes)))
    for c in range(st._n_calls):
        np.testing.assert_array_equal(st._pop_cached(c), ref._pop_cached(c))
    np.testing.assert_array_equal(st._means_host, ref._means_host)
