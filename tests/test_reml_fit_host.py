"""Whole REML fits on CPU: the package's driver against the oracle's fit.

fit_reml reaches the device only through the genotype operator callables
and pcg_solve.  Here the operators are dense CPU kernels and pcg_solve is an
exact dense solve, so the package's evaluation (projection of the fixed
effects, yPy, log|X^T H^-1 X|, affine or multi-component SLQ with its exact
score, AI matrix), its Fisher steps and its line search run in FP32 on CPU
and must reproduce the oracle's FP64 fit: |dh2| < 1e-3 and the
log-likelihood within 1e-4 relative (the tolerances the GPU fits are held
to).  The block PCG itself is checked on the GPU.
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import reml
from oracle import geno as og
from oracle import reml as oreml
from oracle import slq as oslq


def _dense_solve(Hv, B, M=None, tol=1e-2, maxiter=200, X0=None, check_every=2):
    """Exact H X = B with pcg_solve's return contract (X, max_rel_res, iters)."""
    B = torch.as_tensor(B)
    vec = B.ndim == 1
    B2 = (B[:, None] if vec else B).to(torch.float32)
    n = B2.shape[0]
    H = torch.as_tensor(Hv(torch.eye(n, dtype=torch.float32))).double()
    X = torch.linalg.solve(0.5 * (H + H.T), B2.double()).float()
    R = B2.double() - torch.as_tensor(Hv(X)).double()
    den = B2.double().norm(dim=0)
    rel = torch.max(torch.where(den > 0, R.norm(dim=0) / den, torch.zeros_like(den)))
    return (X[:, 0] if vec else X), rel, 1


def _problem(n, m, seed, comps, h2=0.5, n_causal=60):
    rng = np.random.default_rng(seed)
    codes = og.synth_codes(seed, n, np.arange(m))
    mean, inv, _ = og.stats(codes)
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)[None, :]
    Ks, pos = [], 0
    for size in comps:
        Zg = Z[:, pos:pos + size]
        Ks.append(Zg @ Zg.T / float(np.count_nonzero(inv[pos:pos + size] > 0)))
        pos += size
    beta = np.zeros(m)
    idx = rng.choice(m, n_causal, replace=False)
    beta[idx] = rng.normal(size=n_causal)
    g = Z @ beta
    g *= np.sqrt(h2 / np.var(g))
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = (g + rng.normal(scale=np.sqrt(1 - h2), size=n) + X @ [0.5, -0.3]).astype(np.float32)
    return Ks, X, y


def _fit_both(Ks, X, y, *, residual=None, slq_samples=16, slq_m=16, minq_iter=20):
    n = y.size
    G = len(Ks)
    probes = np.random.default_rng(7).choice([-1.0, 1.0], size=(n, slq_samples))
    Kt = [torch.as_tensor(K, dtype=torch.float32) for K in Ks]
    diags = [torch.diagonal(K) for K in Kt]
    param, hist, diag = reml.fit_reml(
        y, tuple(lambda V, K=K: K @ V for K in Kt), diags, X, n_rand_vec=4, maxiter=500,
        minq_iter=minq_iter, slq_samples=slq_samples, slq_m=slq_m, slq_mode="raw",
        pcg_tol=1e-5, verbose=False, return_diagnostics=True, device="cpu",
        slq_probes=torch.as_tensor(probes, dtype=torch.float32),
        residual_diag_list=None if residual is None else [torch.as_tensor(r) for r in residual])
    yo, _, _ = oreml.standardize(y)
    atoms = reml._mean_diag_atoms(diags, n_samples=n)          # FP32 means, as the reference
    kw = dict(diag_atoms=atoms, pcg_tol=1e-6, maxiter=1000)
    if G == 1 and residual is None:
        kw["affine_cache"] = oslq.affine_cache(lambda v: Ks[0] @ v, n, probes, slq_m)
    else:
        kw.update(slq_probes=probes, slq_m=slq_m, residual_diags=residual)
    ctx = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X, **kw)
    po, ho, cur = oreml.fit(ctx, minq_iter=minq_iter)
    ra = (1.0,) if residual is None else np.asarray(residual, np.float64).mean(axis=1)
    h2 = oreml.heritability(param, G, atoms, ra)
    h2_ref = oreml.heritability(po, G, atoms, ra)
    return param, diag, h2, po, cur, h2_ref, hist, ho


@pytest.fixture(autouse=True)
def _exact_solves(monkeypatch):
    monkeypatch.setattr(reml, "pcg_solve", _dense_solve)


def _check(diag, h2, cur, h2_ref, param, po):
    assert abs(h2 - h2_ref) < 1e-3, (h2, h2_ref)
    assert abs(diag["loglik"] - cur["ll"]) <= 1e-4 * abs(cur["ll"]), (diag["loglik"], cur["ll"])
    np.testing.assert_allclose(param, po, rtol=1e-4, atol=1e-6)


def test_single_grm_affine_slq_fit_matches_oracle():
    Ks, X, y = _problem(240, 900, seed=3, comps=[900])
    param, diag, h2, po, cur, h2_ref, hist, ho = _fit_both(Ks, X, y)
    _check(diag, h2, cur, h2_ref, param, po)
    assert 0.2 < h2 < 0.9 and len(hist) >= 2


def test_two_grm_multi_slq_fit_matches_oracle():
    Ks, X, y = _problem(240, 900, seed=5, comps=[400, 500])
    param, diag, h2, po, cur, h2_ref, hist, ho = _fit_both(Ks, X, y, slq_m=12)
    _check(diag, h2, cur, h2_ref, param, po)


def test_two_residual_components_fit_matches_oracle():
    Ks, X, y = _problem(240, 900, seed=9, comps=[900])
    residual = np.stack([np.ones(240), 0.5 + (np.arange(240) % 16) / 16.0])
    param, diag, h2, po, cur, h2_ref, hist, ho = _fit_both(Ks, X, y, residual=residual,
                                                          slq_m=12)
    _check(diag, h2, cur, h2_ref, param, po)
    assert param.size == 3


def test_eight_grm_maf_ld_partition_fit_matches_oracle():
    """The 8-GRM workload's form at a small size: LD-block genotypes, 4 MAF
    bins x 2 LD-score halves, per-component h2 ~ Dirichlet(1) x 0.4."""
    from coherit_gb300 import synth

    n, m = 300, 1600
    codes, maf, _ = synth.ld_block_genotypes(21, n, m, block=200)
    groups = synth.maf_ld_partition(maf, synth.block_ld_scores(codes, block=200))
    h2s = synth.dirichlet_h2(21, 8, total=0.4)
    y, X = synth.partitioned_phenotype(codes, groups, h2s, seed=21, n_causal_per=25, n_covar=1)
    mean, inv, _ = og.stats(codes)
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)[None, :]
    Ks = [Z[:, g] @ Z[:, g].T / float(np.count_nonzero(inv[g] > 0)) for g in groups]
    param, diag, h2, po, cur, h2_ref, hist, ho = _fit_both(Ks, X, y, slq_m=12)
    _check(diag, h2, cur, h2_ref, param, po)
    assert param.size == 9 and len(hist) >= 2


def test_scoring_optimizer_fit_matches_oracle_scoring_fit():
    """optimizer="smile_scoring" with the phenotype and 64 Rademacher trace
    probes as one 67-column right-hand-side block ([X | y | probes]): the
    package's one-trial scoring driver (Taylor log-determinants, Hutchinson
    traces from the probe columns of the solves) against the oracle's
    restatement of the same driver, on the same probes."""
    Ks, X, y = _problem(200, 800, seed=13, comps=[800])
    n = y.size
    slq = np.random.default_rng(7).choice([-1.0, 1.0], size=(n, 16))
    tp = np.random.default_rng(8).choice([-1.0, 1.0], size=(n, 64))
    Kt = torch.as_tensor(Ks[0], dtype=torch.float32)
    diags = [torch.diagonal(Kt)]
    param, hist, diag = reml.fit_reml(
        y, (lambda V: Kt @ V,), diags, X, n_rand_vec=64, maxiter=500, minq_iter=30,
        slq_samples=16, slq_m=16, pcg_tol=1e-5, verbose=False, return_diagnostics=True,
        device="cpu", optimizer="smile_scoring",
        slq_probes=torch.as_tensor(slq, dtype=torch.float32),
        trace_probes=torch.as_tensor(tp, dtype=torch.float32))
    yo, _, _ = oreml.standardize(y)
    atoms = reml._mean_diag_atoms(diags, n_samples=n)
    ctx = oreml.Context(yo, [lambda v: Ks[0] @ v], X, diag_atoms=atoms, pcg_tol=1e-6,
                        maxiter=1000, trace_probes=tp,
                        affine_cache=oslq.affine_cache(lambda v: Ks[0] @ v, n, slq, 16))
    po, ho, cur = oreml.fit_scoring(ctx, minq_iter=30)
    h2 = oreml.heritability(param, 1, atoms)
    h2_ref = oreml.heritability(po, 1, atoms)
    assert abs(h2 - h2_ref) < 1e-3, (h2, h2_ref)
    assert abs(diag["loglik"] - cur["ll"]) <= 1e-4 * abs(cur["ll"])
    # Same trajectory step by step, Taylor steps included.  On this problem
    # both settle into the same period-3 cycle (full, full, Taylor) and stop
    # at the iteration limit: the reference's scoring loop has no other exit
    # while the step stays above scoring_step_tol.
    assert len(hist) == len(ho) == 30
    assert [h["slq_taylor"] for h in hist] == [h["taylor"] for h in ho]
    for h, o in zip(hist, ho):
        np.testing.assert_allclose(h["params"], o["params"], rtol=1e-4)
