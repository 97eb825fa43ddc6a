"""Rare-variant sparse operator on the GPU versus the oracle (GPU).

* The entries built on the device from BED bytes (two chunked passes, keep
  list, chunks that split the file) equal the oracle's entry lists exactly,
  and the FP32 statistics are bit-exact.
* K V, X^T V and theta_g K V + theta_e V are within 1e-5 (relative, per
  column) of the FP64 oracle for every lane layout (k = 1 .. 80, including
  widths that are not multiples of 4).
* The sparse and the dense (tensor-core) streamer built from the same BED
  give the same operator, the same standardised columns (bit-exact) and the
  same exact diagonal.
* A fit with one dense and one rare-variant GRM matches the FP64 oracle fit
  (|delta h2| < 1e-3).
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import synth
from coherit_gb300.bed import write_bed
from coherit_gb300.geno_stream import ArraySource, GenoBlockStreamer
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter
from coherit_gb300.sparse_stream import SparseGenoBlockStreamer, SyntheticRareSource
from oracle import geno as og
from oracle import reml as oreml
from oracle import sparse12 as osp

pytestmark = pytest.mark.gpu


def _codes(seed, n, m, missing=0.01):
    codes = osp.rare_codes(seed, n, m, maf_lo=0.0005, maf_hi=0.03, missing=missing)
    codes[:, 0] = 0
    codes[:, 1] = osp.MISS
    codes[:, 2] = 1
    return codes


def _bed(tmp_path, codes, name="r"):
    prefix = str(tmp_path / name)
    write_bed(prefix, np.where(codes == 3, -1, codes.astype(np.int16)))
    return prefix


def _as_int8(codes):
    g = codes.astype(np.int8)
    g[codes == 3] = -127
    return g


def _rel(a, b):
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


@pytest.mark.parametrize("mask,chunk", [(False, None), (True, None), (False, 7)])
def test_bed_entries_and_stats(cuda, tmp_path, monkeypatch, mask, chunk):
    n, m = 2049, 600
    codes = _codes(31, n, m)
    prefix = _bed(tmp_path, codes)
    keep = np.random.default_rng(4).random(n) < 0.7 if mask else None
    if chunk is not None:
        monkeypatch.setenv("COHERIT_BED_CHUNK_BYTES", str(chunk * ((n + 3) // 4)))
    st = SparseGenoBlockStreamer(bed_prefix=prefix, sample_mask=keep, call_width=256)
    sub = codes if keep is None else codes[keep]
    col_off, rows, vals = st.read_entries()
    ref = osp.csc_from_codes(sub)
    np.testing.assert_array_equal(col_off, ref[0])
    np.testing.assert_array_equal(rows, ref[1])
    np.testing.assert_array_equal(vals, ref[2])
    s = osp.bed_counts_stats(sub)
    np.testing.assert_array_equal(st._means_host, s["mean"])
    np.testing.assert_array_equal(st._inv_sds_host, s["inv"])
    assert st._eff_m_host == s["eff"]
    assert st._mean_diag_atom_host == pytest.approx(s["atom"], rel=1e-12)
    meta = st.sparse_block_metadata()
    assert len(meta) == st._n_calls == len(st.block_backend_plan())
    assert sum(d["nnz_het"] for d in meta) == int((sub == 1).sum())
    assert sum(d["nnz_miss"] for d in meta) == int((sub == 3).sum())
    # The in-memory source path builds the same entries.
    st2 = SparseGenoBlockStreamer(ArraySource(_as_int8(sub)), call_width=256)
    for a, b in zip(st2.read_entries(), (col_off, rows, vals)):
        np.testing.assert_array_equal(a, b)
    st.close()
    st2.close()


def test_synthetic_generator_matches_oracle(cuda):
    """The device generator writes exactly the oracle's genotypes; the host
    source path (forced by a sample mask) builds the same entries."""
    n, m = 1500, 700
    src = SyntheticRareSource(n, m, seed=12, maf_range=(0.001, 0.04), missing_rate=0.01)
    st = SparseGenoBlockStreamer(src)
    codes = osp.synth_rare_codes(12, n, np.arange(m), *src.maf_range_q24,
                                 missing_q24=src.missing_q24)
    ref = osp.csc_from_codes(codes)
    for a, b in zip(st.read_entries(), ref):
        np.testing.assert_array_equal(a, b)
    st2 = SparseGenoBlockStreamer(src, sample_mask=np.ones(n, dtype=bool))
    for a, b in zip(st2.read_entries(), ref):
        np.testing.assert_array_equal(a, b)
    st.close()
    st2.close()


@pytest.mark.parametrize("k", [1, 3, 4, 5, 8, 13, 16, 31, 32, 48, 64, 80])
def test_operator_matches_fp64_oracle(cuda, tmp_path, k):
    n, m = 3000, 2500
    codes = _codes(40 + k, n, m)
    st = SparseGenoBlockStreamer(bed_prefix=_bed(tmp_path, codes))
    mean, inv = st._means_host, st._inv_sds_host
    csc = osp.csc_from_codes(codes)
    V = np.random.default_rng(k).normal(size=(n, k)).astype(np.float32) + 0.25
    Vd = torch.as_tensor(V, device=cuda)
    ref = osp.kv_f64(*csc, mean, inv, V, st._eff_m_host)
    assert _rel(st.kv(Vd).cpu().numpy(), ref) < 1e-5
    xt = osp.xtv_f64(*csc, mean, inv, V)
    assert _rel(st.xtv(Vd).cpu().numpy(), xt) < 1e-5
    assert _rel(st.xtv(Vd, normalize=True).cpu().numpy(), xt / st._eff_m_host) < 1e-5
    hv = st.weighted_component_hv([0.7], 0.3, Vd).cpu().numpy()
    assert _rel(hv, 0.7 * ref + 0.3 * V) < 1e-5
    st.close()


def test_unaligned_strided_input(cuda, tmp_path):
    """A right-hand side whose rows are not 16-byte aligned takes the scalar
    load path and gives the same result."""
    n, m, k = 1500, 900, 6
    codes = _codes(77, n, m)
    st = SparseGenoBlockStreamer(bed_prefix=_bed(tmp_path, codes))
    V = torch.randn((n, k), device=cuda, generator=torch.Generator("cuda").manual_seed(3))
    a = st.kv(V).cpu().numpy()
    ref = osp.kv_f64(*osp.csc_from_codes(codes), st._means_host, st._inv_sds_host,
                     V.cpu().numpy(), st._eff_m_host)
    assert _rel(a, ref) < 1e-5
    v1 = V[:, 2].contiguous()
    np.testing.assert_allclose(st.kv(v1).cpu().numpy(), st.kv(V[:, 2:3]).cpu().numpy()[:, 0],
                               rtol=1e-6, atol=1e-6)
    st.close()


def test_sparse_and_dense_streamers_agree(cuda, tmp_path):
    n, m = 2500, 3000
    codes = _codes(91, n, m)
    prefix = _bed(tmp_path, codes)
    sp = SparseGenoBlockStreamer(bed_prefix=prefix)
    de = GenoBlockStreamer(bed_prefix=prefix, precision="bf16x3")
    np.testing.assert_array_equal(sp._means_host, de._means_host)
    np.testing.assert_array_equal(sp._inv_sds_host, de._inv_sds_host)
    assert sp._eff_m_host == de._eff_m_host
    assert sp._mean_diag_atom_host == pytest.approx(de._mean_diag_atom_host, rel=1e-12)
    V = torch.randn((n, 16), device=cuda, generator=torch.Generator("cuda").manual_seed(5))
    a, b = sp.kv(V).cpu().numpy(), de.kv(V).cpu().numpy()
    assert _rel(a, b) < 2e-5
    idx = np.asarray([0, 1, 2, 5, 17, 2999, 5])
    np.testing.assert_array_equal(sp.extract_standardized_columns(idx),
                                  de.extract_standardized_columns(idx))
    with pytest.raises(IndexError):
        sp.standardized_columns([m])
    np.testing.assert_allclose(sp.exact_diag().cpu().numpy(), de.exact_diag().cpu().numpy(),
                               rtol=1e-6, atol=1e-7)
    U = torch.randn((n, 12), device=cuda, generator=torch.Generator("cuda").manual_seed(6))
    core = sp.build_projected_core_atom(U).cpu().numpy()
    ref = osp.projected_core_atom_f64(*osp.csc_from_codes(codes), sp._means_host,
                                      sp._inv_sds_host, U.cpu().numpy(), sp._eff_m_host)
    np.testing.assert_allclose(core, ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
    sp.close()
    de.close()


def test_exact_diag_matches_oracle(cuda, tmp_path):
    n, m = 1200, 800
    codes = _codes(95, n, m, missing=0.05)
    st = SparseGenoBlockStreamer(bed_prefix=_bed(tmp_path, codes))
    ref = og.exact_diag(codes, st._means_host, st._inv_sds_host, st._eff_m_host)
    np.testing.assert_allclose(st.exact_diag().cpu().numpy(), ref, rtol=1e-6)
    st.close()


def test_no_valid_snps(cuda, tmp_path):
    n, m = 100, 3
    codes = np.zeros((n, m), dtype=np.uint8)
    codes[:, 1] = osp.MISS
    codes[:, 2] = 1
    st = SparseGenoBlockStreamer(ArraySource(_as_int8(codes)))
    assert st._eff_m_host == 0.0
    V = torch.ones((n, 3), device=cuda)
    np.testing.assert_array_equal(st.kv(V).cpu().numpy(), np.zeros((n, 3), np.float32))
    np.testing.assert_array_equal(st.xtv(V).cpu().numpy(), np.zeros((m, 3), np.float32))
    np.testing.assert_array_equal(st.weighted_component_hv([1.0], 2.0, V).cpu().numpy(),
                                  2.0 * np.ones((n, 3), np.float32))
    st.close()


def test_dense_plus_rare_fit_matches_oracle(cuda, tmp_path):
    """One common-variant GRM (dense tensor-core streamer) and one
    rare-variant GRM (sparse streamer), as the reference appends rare
    streamers after the dense ones."""
    n, m_common, m_rare = 900, 3000, 6000
    common = og.synth_codes(51, n, np.arange(m_common))
    rare = _codes(52, n, m_rare, missing=0.0)
    rng = np.random.default_rng(53)
    b_c = rng.normal(size=m_common) * (rng.random(m_common) < 0.05)
    b_r = rng.normal(size=m_rare) * (rng.random(m_rare) < 0.05)
    mc, ic, _ = og.stats(common)
    mr, ir, _ = og.stats(rare)
    g = og.zxb_f64(common, mc, ic, b_c) + 2.0 * og.zxb_f64(rare, mr, ir, b_r)
    y = g / g.std() * np.sqrt(0.5) + rng.normal(size=n) * np.sqrt(0.5)
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    cfg = FitConfig(sources=[ArraySource(_as_int8(common))],
                    rare_bed_prefix=_bed(tmp_path, rare, "rare"), slq_samples=16, slq_m=16,
                    precond_rank=64, reml_pcg_tol=1e-5, minq_iter=15, max_pcg_iters=500,
                    slq_mode="raw")
    fitter = InfinitesimalREMLFitter(cfg)
    assert fitter._has_sparse and fitter._n_dense_streamers == 1
    probes = np.random.default_rng(9).choice([-1.0, 1.0], size=(n, 16))
    res = fitter.fit_infinitesimal(y, X, slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    sp = fitter.streamers[1]
    de = fitter.streamers[0]
    Zc = og.diff_f64(common, de._means_host) * de._inv_sds_host.astype(np.float64)[None, :]
    Kc = Zc @ Zc.T / de._eff_m_host
    Zr = og.diff_f64(rare, sp._means_host) * sp._inv_sds_host.astype(np.float64)[None, :]
    Kr = Zr @ Zr.T / sp._eff_m_host
    yo, _, _ = oreml.standardize(y)
    atoms = np.asarray([de._mean_diag_atom_host, sp._mean_diag_atom_host])
    ctx_o = oreml.Context(yo, [lambda v: Kc @ v, lambda v: Kr @ v], X, diag_atoms=atoms,
                          slq_probes=probes, slq_m=16, pcg_tol=1e-5, maxiter=500)
    po, _, _ = oreml.fit(ctx_o, minq_iter=15)
    h2_ref = oreml.heritability(po, 2, atoms)
    assert abs(res.heritability - h2_ref) < 1e-3, (res.heritability, h2_ref)
    # Effects of the rare component come from its X^T alpha (reml_model.py:1495-1523).
    eff = fitter.estimate_effects(y, var_components=res.var_components, covar=X)
    assert len(eff.snp_effects) == 2 and eff.snp_effects[1].shape[0] == m_rare
    with pytest.raises(NotImplementedError):
        fitter.predict(eff, test_fitter=fitter)
    for s in fitter.streamers:
        s.close()


@pytest.mark.parametrize("merged_float", [False, True])
def test_kv_impl_shard_functions(cuda, merged_float):
    """sparse_kv_shard / sparse_xtv_shard / sparse_projected_core_atom_shard
    on a shard payload (host arrays with the shard's own statistics), as the
    reference's sparse streamer passes them (kv_impl.py:823-905)."""
    from coherit_gb300 import kv_impl

    n, m = 2000, 900
    codes = _codes(61, n, m, missing=0.02)
    col_off, rows, vals = osp.csc_from_codes(codes)
    mean, inv, _ = og.stats(codes)
    cols = np.repeat(np.arange(m), np.diff(col_off)).astype(np.int32)
    if merged_float:
        v, _ = osp.entry_values(col_off, vals, mean)
        vals_in = v.astype(np.float32)
    else:
        vals_in = vals
    pay = osp.shard_payload(col_off, rows, vals, mean, inv, n)
    V = np.random.default_rng(3).normal(size=(n, 7)).astype(np.float32) + 0.2
    Vd = torch.as_tensor(V, device=cuda)
    got = kv_impl.sparse_kv_shard(
        Vd, n=n, m=m, sum_v=Vd.sum(0), mean=mean, b=pay["b"].astype(np.float32),
        inv_sq=(inv.astype(np.float32) ** 2), row_b=pay["row_b"].astype(np.float32),
        sum_a0_sq=np.float32(pay["sum_a0_sq"]), csc_all_rows=rows, csc_all_cols=cols,
        csc_all_vals=vals_in).cpu().numpy()
    ref = osp.kv_f64(col_off, rows, vals, mean, inv, V)
    assert _rel(got, ref) < 1e-5
    xt = kv_impl.sparse_xtv_shard(Vd, m=m, mean=mean, inv=inv, csc_all_rows=rows,
                                  csc_all_cols=cols, csc_all_vals=vals_in).cpu().numpy()
    assert _rel(xt, osp.xtv_f64(col_off, rows, vals, mean, inv, V)) < 1e-5
    core = kv_impl.sparse_projected_core_atom_shard(
        Vd, m=m, mean=mean, inv=inv, csc_all_rows=rows, csc_all_cols=cols,
        csc_all_vals=vals_in).cpu().numpy()
    cref = osp.projected_core_atom_f64(col_off, rows, vals, mean, inv, V, 1.0,
                                       subtract_identity=False)
    np.testing.assert_allclose(core, cref, rtol=1e-4, atol=1e-4 * np.abs(cref).max())
