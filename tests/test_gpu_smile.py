"""SMILE block-weighted GRM operator (GPU) against the FP64 oracle.

Tolerances: operator products, diagonals and SNP effects within 1e-5
relative per column of FP64 (the W products run in FP32 as in the
reference); normaliser within 1e-6 relative; standardised columns
bit-exact against the reference's FP32 formula; REML |delta h2| < 1e-3.
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import synth
from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
from coherit_gb300.reml import fit_reml
from coherit_gb300.smile_block_w import (SmileBlockWeightedOperator,
                                         SmileMultiBlockWeightedOperator)
from oracle import geno as og
from oracle import reml as oreml
from oracle import slq as oslq
from oracle import smile as osm

pytestmark = pytest.mark.gpu
TOL = 1e-5


def col_rel(out, ref):
    out = np.asarray(out, np.float64).reshape(len(ref), -1)
    ref = np.asarray(ref, np.float64).reshape(len(ref), -1)
    return float(np.max(np.linalg.norm(out - ref, axis=0) /
                        np.maximum(np.linalg.norm(ref, axis=0), 1e-300)))


def wishart(rng, p):
    X = rng.normal(size=(p, p))
    return (X @ X.T / p).astype(np.float32)


def _setup(n, m, seed, miss=0.0):
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=seed, missing_rate=miss), precision="bf16x3")
    codes = og.synth_codes(seed, n, np.arange(m), missing_q24=synth.missing_rate_q24(miss))
    return st, codes


def test_standardized_columns_bit_exact(cuda):
    st, codes = _setup(300, 900, seed=61, miss=0.03)
    idx = np.array([0, 5, 899, 450, 5, 128, 127])
    got = st.extract_standardized_columns(idx)
    ref = osm.standardized_fp32(codes[:, idx], st._means_host[idx], st._inv_sds_host[idx])
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("diag_mode", ["full", "mean"])
def test_smile_operator_matches_oracle(cuda, diag_mode):
    n, m = 400, 1500
    st, codes = _setup(n, m, seed=62, miss=0.01)
    rng = np.random.default_rng(1)
    Ws = [wishart(rng, 500), wishart(rng, 700), wishart(rng, 300)]
    op = SmileBlockWeightedOperator(st, Ws, diag_mode=diag_mode)
    Z = osm.standardized(codes, st._means_host, st._inv_sds_host)
    ok = osm.SmileKernel(Z, [(0, Ws[0]), (500, Ws[1]), (1200, Ws[2])])
    assert abs(op.normalizer - ok.c) <= 1e-6 * ok.c
    V = rng.normal(size=(n, 5)).astype(np.float32)
    assert col_rel(op.kv(V).cpu().numpy(), ok.kv(V)) < TOL
    assert col_rel(op.kv(V[:, 0]).cpu().numpy(), ok.kv(V[:, :1])) < TOL
    assert col_rel(op.block_kv(V, 1).cpu().numpy(), ok.kv(V, block_idx=1)) < TOL
    stacked = op.stacked_block_kv(V).cpu().numpy()
    assert stacked.shape == (3, n, 5)
    assert col_rel(stacked.sum(0), ok.kv(V)) < TOL
    assert col_rel(op.weighted_hv(0.7, 0.4, V).cpu().numpy(), ok.weighted_hv(0.7, 0.4, V)) < TOL
    beta = op.snp_effects(V[:, 2], np.array([0.7])).cpu().numpy()
    assert col_rel(beta, ok.snp_effects(V[:, 2], 0.7)) < TOL
    if diag_mode == "full":
        assert col_rel(op.diag().cpu().numpy(), ok.diag_full()) < TOL
    else:
        assert abs(float(op.diag()) - ok.diag_mean()) < 1e-6
    with pytest.raises(IndexError):
        op.block_kv(V, 3)


def test_identity_operator_is_the_grm(cuda):
    n, m = 350, 1300
    st, codes = _setup(n, m, seed=63)
    op = SmileBlockWeightedOperator.identity(st, block_size=256)
    assert op.n_blocks == 6
    # Without missing genotypes tr(Z Z^T)/n = m_eff, so K is the plain GRM.
    assert abs(op.normalizer - st._eff_m_host) <= 1e-5 * st._eff_m_host
    V = np.random.default_rng(2).normal(size=(n, 4)).astype(np.float32)
    assert col_rel(op.kv(V).cpu().numpy(), st.kv(V).cpu().numpy()) < 1e-5
    op_rank = SmileBlockWeightedOperator.identity(st, block_size=256,
                                                  normalization="effective_rank")
    assert op_rank.normalizer == float(m)


def test_coverage_and_validation_errors(cuda):
    st, _ = _setup(200, 600, seed=64)
    rng = np.random.default_rng(3)
    with pytest.raises(ValueError, match="cover"):
        SmileBlockWeightedOperator(st, [wishart(rng, 500)])
    with pytest.raises(ValueError, match="exceeds"):
        SmileBlockWeightedOperator(st, [wishart(rng, 500), wishart(rng, 200)])
    with pytest.raises(ValueError, match="effective rank"):
        SmileBlockWeightedOperator(st, [wishart(rng, 600)], normalization="effective_rank")
    op = SmileBlockWeightedOperator(st, [wishart(rng, 600)], normalization="effective_rank",
                                    effective_ranks=[450.0])
    assert op.normalizer == 450.0
    op2 = SmileBlockWeightedOperator(st, [wishart(rng, 100)], strict_coverage=False,
                                     start_offsets=[250])
    assert op2.blocks[0].start == 250


def test_multi_grm_shares_one_xtv(cuda):
    n, m = 300, 1000
    st, codes = _setup(n, m, seed=65)
    rng = np.random.default_rng(4)
    groups = [[wishart(rng, 400), wishart(rng, 200)], [wishart(rng, 400)]]
    mop = SmileMultiBlockWeightedOperator.from_weight_matrix_groups(st, groups)
    assert mop.n_grm == 2
    Z = osm.standardized(codes, st._means_host, st._inv_sds_host)
    k0 = osm.SmileKernel(Z, [(0, groups[0][0]), (400, groups[0][1])])
    k1 = osm.SmileKernel(Z, [(600, groups[1][0])])
    V = rng.normal(size=(n, 3)).astype(np.float32)
    assert col_rel(mop.kv(V, 1).cpu().numpy(), k1.kv(V)) < TOL
    stacked = mop.stacked_kv(V).cpu().numpy()
    assert col_rel(stacked[0], k0.kv(V)) < TOL and col_rel(stacked[1], k1.kv(V)) < TOL
    got = mop.weighted_hv(np.array([0.3, 1.2]), 0.5, V).cpu().numpy()
    assert col_rel(got, osm.multi_weighted_hv([k0, k1], [0.3, 1.2], 0.5, V)) < TOL
    with pytest.raises(ValueError):
        mop.weighted_hv(np.array([0.3]), 0.5, V)


def test_smile_reml_fit_matches_oracle(cuda):
    n, m = 800, 3000
    st, codes = _setup(n, m, seed=66)
    rng = np.random.default_rng(5)
    Ws = [wishart(rng, 500) for _ in range(6)]
    op = SmileBlockWeightedOperator(st, Ws, diag_mode="mean")
    Z = osm.standardized(codes, st._means_host, st._inv_sds_host)
    ok = osm.SmileKernel(Z, [(500 * i, W) for i, W in enumerate(Ws)])
    K = ok.dense()
    y, X, _, _ = synth.phenotype(66, n, m, h2=0.5, n_causal=300, n_covar=2)
    probes = rng.choice([-1.0, 1.0], size=(n, 30))
    param, _, d = fit_reml(y, [op.kv], [op.diag()], X, n_rand_vec=30, maxiter=500,
                           minq_iter=20, slq_samples=30, slq_m=30, pcg_tol=1e-6, verbose=False,
                           weighted_hv=op.weighted_hv, return_diagnostics=True,
                           slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    yo, _, _ = oreml.standardize(y)
    cache = oslq.affine_cache(lambda v: K @ v, n, probes, 30)
    ctx = oreml.Context(yo, [lambda v: K @ v], X, diag_atoms=[ok.diag_mean()],
                        affine_cache=cache, pcg_tol=1e-6, maxiter=500)
    po, _, _ = oreml.fit(ctx, minq_iter=20)
    h2 = oreml.heritability(param, 1, [ok.diag_mean()])
    h2o = oreml.heritability(po, 1, [ok.diag_mean()])
    assert abs(h2 - h2o) < 1e-3, (h2, h2o)


def test_fitter_with_smile_groups_matches_oracle(cuda):
    """Two SMILE GRMs through FitConfig (matrix groups), projected-core
    preconditioner from the SMILE kernels, against the FP64 oracle fit."""
    from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter

    n, m = 700, 3000
    st, codes = _setup(n, m, seed=67)
    rng = np.random.default_rng(6)
    groups = [[wishart(rng, 500) for _ in range(3)], [wishart(rng, 500) for _ in range(3)]]
    y, X, _, _ = synth.phenotype(67, n, m, h2=0.4, n_causal=300, n_covar=2)
    cfg = FitConfig(slq_samples=16, slq_m=16, precond_rank=64, reml_pcg_tol=1e-5, minq_iter=15,
                    max_pcg_iters=500, slq_mode="raw", smile_weight_matrix_groups=groups)
    fitter = InfinitesimalREMLFitter(cfg, [st])
    probes = rng.choice([-1.0, 1.0], size=(n, 16))
    res = fitter.fit_infinitesimal(y, X, slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    Z = osm.standardized(codes, st._means_host, st._inv_sds_host)
    ks = [osm.SmileKernel(Z, [(500 * i, W) for i, W in enumerate(groups[0])]),
          osm.SmileKernel(Z, [(1500 + 500 * i, W) for i, W in enumerate(groups[1])])]
    Ks = [k.dense() for k in ks]
    atoms = np.asarray([k.diag_mean() for k in ks])
    yo, _, _ = oreml.standardize(y)
    ctx_o = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X, diag_atoms=atoms,
                          slq_probes=probes, slq_m=16, pcg_tol=1e-5, maxiter=500)
    po, _, _ = oreml.fit(ctx_o, minq_iter=15)
    h2_ref = oreml.heritability(po, 2, atoms)
    assert abs(res.heritability - h2_ref) < 1e-3, (res.heritability, h2_ref)
    with pytest.raises(ValueError, match="only one SMILE"):
        InfinitesimalREMLFitter(FitConfig(smile_identity=True, smile_weight_matrix_groups=groups),
                                [st])
