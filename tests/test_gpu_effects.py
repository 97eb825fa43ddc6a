"""Effect estimation, prediction and batched H^{-1} solves on the GPU
operator, against FP64 dense algebra on the same genotypes.

Tolerances: fixed effects, BLUP random effects, SNP effects, predictions
and H^{-1} B within 1e-5 relative (PCG tol 1e-6; H has condition
number ~3 here, so the solution error stays near 3e-6)."""
import numpy as np
import pytest
import torch

from coherit_gb300 import synth
from coherit_gb300.geno_stream import ArraySource, GenoBlockStreamer
from coherit_gb300.hinv import solve_hinv_columns_batched
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter
from oracle import geno as og
from oracle import reml as oreml
from oracle import smile as osm

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _codes(seed, n, m, miss=0.0):
    return og.synth_codes(seed, n, np.arange(m), missing_q24=synth.missing_rate_q24(miss))


def _array_streamer(codes, comps=None):
    g = codes.astype(np.int8)
    g[codes == 3] = -127
    return GenoBlockStreamer(ArraySource(g), component_block_sizes=comps, precision="bf16x3")


def _oracle_effects(Zs, effs, theta, y, X):
    n = Zs[0].shape[0]
    Ks = [Z @ Z.T / e for Z, e in zip(Zs, effs)]
    H = sum(t * K for t, K in zip(theta[:-1], Ks)) + theta[-1] * np.eye(n)
    ys, ym, ysc = oreml.standardize(y)
    Hy = np.linalg.solve(H, ys)
    HX = np.linalg.solve(H, X)
    fixed = np.linalg.solve(X.T @ HX, X.T @ Hy)
    alpha = Hy - HX @ fixed
    comps = [t * (K @ alpha) for t, K in zip(theta[:-1], Ks)]
    snps = [t / e * (Z.T @ alpha) for t, Z, e in zip(theta[:-1], Zs, effs)]
    return fixed, alpha, comps, snps, ym, ysc, H


@pytest.mark.parametrize("comps", [None, [900, 1100]])
def test_effects_and_prediction_match_dense(cuda, comps):
    n_tr, n_te, m = 500, 200, 2000
    codes = _codes(71, n_tr + n_te, m, miss=0.01)
    st_tr = _array_streamer(codes[:n_tr], comps)
    st_te = _array_streamer(codes[n_tr:], comps)
    y, X, _, _ = synth.phenotype(71, n_tr + n_te, m, h2=0.5, n_causal=200, n_covar=2,
                                 missing_q24=synth.missing_rate_q24(0.01))
    cfg = FitConfig(precond_rank=32, effect_pcg_tol=1e-6, max_pcg_iters=1000,
                    vc_block_sizes=comps)
    fitter = InfinitesimalREMLFitter(cfg, [st_tr])
    G = 1 if comps is None else 2
    theta = np.array([0.3, 0.25, 0.5][-(G + 1):]) if G == 2 else np.array([0.45, 0.55])
    eff = fitter.estimate_effects(y[:n_tr], var_components=theta, covar=X[:n_tr])
    Z = osm.standardized(codes[:n_tr], st_tr._means_host, st_tr._inv_sds_host)
    if comps is None:
        Zs, effs = [Z], [st_tr._eff_m_host]
    else:
        Zs = [Z[:, :comps[0]], Z[:, comps[0]:]]
        effs = list(st_tr._component_eff_m_host.astype(np.float64))
    fixed, alpha, rcomps, snps, ym, ysc, _ = _oracle_effects(Zs, effs, theta, y[:n_tr], X[:n_tr])
    assert rel(eff.fixed_effects.cpu(), fixed) < 1e-5
    assert rel(eff.random_effect.cpu(), sum(rcomps)) < 1e-5
    for g in range(G):
        assert rel(eff.random_effect_components[g].cpu(), rcomps[g]) < 1e-5
        assert rel(eff.snp_effects[g].cpu(), snps[g]) < 1e-5
    test = InfinitesimalREMLFitter(FitConfig(vc_block_sizes=comps, precond_rank=0), [st_te])
    pred = fitter.predict(eff, test_fitter=test, test_covar=X[n_tr:])
    Zt = osm.standardized(codes[n_tr:], st_tr._means_host, st_tr._inv_sds_host)
    beta = np.concatenate(snps)
    y_std = X[n_tr:].astype(np.float64) @ fixed + Zt @ beta
    assert rel(pred.y_pred_std.cpu(), y_std) < 1e-5
    assert rel(pred.y_pred.cpu(), ym + ysc * y_std) < 1e-5
    with pytest.raises(ValueError, match="covariates"):
        fitter.predict(eff, test_fitter=test, test_covar=None)


def test_batched_hinv_solves(cuda):
    n, m = 400, 1500
    codes = _codes(72, n, m)
    st = _array_streamer(codes)
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=0), [st])
    ops = fitter._assemble_reml_operators()
    theta_g, theta_e = np.array([0.6]), 0.4
    hv = fitter._make_hv(ops, theta_g, theta_e)
    Z = osm.standardized(codes, st._means_host, st._inv_sds_host)
    H = theta_g[0] * (Z @ Z.T) / st._eff_m_host + theta_e * np.eye(n)
    B = np.random.default_rng(1).normal(size=(n, 150)).astype(np.float32)
    X, diag = solve_hinv_columns_batched(hv=hv, precond=None, rhs=B, warm_start=None, tol=1e-6,
                                         maxiter=500, batch_size=64, stage="test")
    assert isinstance(X, np.ndarray) and diag["n_batches"] == 3
    ref = np.linalg.solve(H, B.astype(np.float64))
    assert rel(X, ref) < 1e-5
    Xd, _ = solve_hinv_columns_batched(hv=hv, precond=None, rhs=torch.as_tensor(B, device="cuda"),
                                       warm_start=torch.as_tensor(X, device="cuda"), tol=1e-6,
                                       maxiter=500, batch_size=80, stage="test")
    assert Xd.is_cuda and rel(Xd.cpu(), ref) < 1e-5
    with pytest.raises(RuntimeError, match="did not converge"):
        solve_hinv_columns_batched(hv=hv, precond=None, rhs=B[:, :4], warm_start=None, tol=1e-9,
                                   maxiter=1, batch_size=4, stage="screen")


# tests/test_sparse_reml_regressions.py:437-455 of the reference
def test_hinv_column_batches_bound_rhs_and_match_exact_solution(cuda):
    rhs = np.arange(35, dtype=np.float32).reshape(7, 5) + 1.0
    X, diag = solve_hinv_columns_batched(hv=lambda v: 2.0 * v, precond=lambda v: 0.5 * v, rhs=rhs,
                                         warm_start=np.zeros_like(rhs), tol=1e-6, maxiter=10,
                                         batch_size=2, stage="unit test")
    np.testing.assert_allclose(X, rhs / 2.0, rtol=1e-6, atol=1e-6)
    assert (diag["n_batches"], diag["n_columns"], diag["batch_size"]) == (3, 5, 2)
    assert diag["max_iterations"] <= 2


# tests/test_sparse_reml_regressions.py:458-473 of the reference
def test_hinv_warm_hit_checks_the_true_residual_once_per_batch(cuda):
    rhs = np.arange(35, dtype=np.float32).reshape(7, 5) + 1.0
    calls = []

    def hv(v):
        calls.append(v.shape[1])
        return 2.0 * v

    X, diag = solve_hinv_columns_batched(hv=hv, precond=None, rhs=rhs, warm_start=rhs / 2.0,
                                         tol=1e-6, maxiter=10, batch_size=2, stage="warm-hit test")
    np.testing.assert_array_equal(X, rhs / 2.0)
    assert calls == [2, 2, 1]
    assert diag["total_batch_iterations"] == 0
    assert diag["max_true_relative_residual"] == 0.0
