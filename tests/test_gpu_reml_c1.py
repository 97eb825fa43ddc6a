"""The small CPU-runnable single-GRM configuration, exactly as specified, fitted
on the GPU operator and checked against the FP64 oracle on the same genotypes
and probes.

Configuration: n=2000 samples x m=10000 SNPs from the MAF~U(0.05,0.5)/HWE
generator with seed 0; phenotype from 1000 causal SNPs with N(0,1) effects
scaled to h2=0.5 plus N(0, 0.5) noise; covariates X = [1, 2 x N(0,1)]; 30
Rademacher probes, 30 Lanczos steps, PCG tol 1e-6.

Tolerances: |delta h2| < 1e-3; log-likelihood, log-determinant and
Hutchinson traces within 1e-4 relative.
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import reml as greml
from coherit_gb300 import synth
from coherit_gb300.configs import C1
from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
from oracle import geno as og
from oracle import reml as oreml
from oracle import slq as oslq

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1():
    n, m = C1.n, C1.m
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=C1.seed), precision="bf16x3")
    codes = og.synth_codes(C1.seed, n, np.arange(m))
    y, X, _, _ = synth.phenotype(C1.seed, n, m, h2=C1.h2, n_causal=C1.n_causal,
                                 n_covar=C1.n_covar, noise_var=0.5)
    mean, inv = st._means_host, st._inv_sds_host
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)[None, :]
    K = Z @ Z.T / float(st._eff_m_host)
    atoms = [float(st._mean_diag_atom_host)]
    yield st, K, y, X, atoms
    st.close()


def _oracle_ctx(K, y, X, atoms, slq_probes, trace_probes=None):
    n = y.size
    yo, _, _ = oreml.standardize(y)
    cache = oslq.affine_cache(lambda v: K @ v, n, slq_probes, C1.slq_m)
    return oreml.Context(yo, [lambda v: K @ v], X, diag_atoms=atoms, affine_cache=cache,
                         pcg_tol=C1.pcg_tol, maxiter=1000, trace_probes=trace_probes)


def test_c1_strict_fit_matches_oracle(cuda, c1):
    st, K, y, X, atoms = c1
    n = y.size
    probes = np.random.default_rng(C1.seed).choice([-1.0, 1.0], size=(n, C1.slq_samples))
    param, hist, diag = greml.fit_reml(
        y, [lambda V: st.kv(V)], [st.diag()], X, n_rand_vec=30, maxiter=1000,
        minq_iter=C1.minq_iter, slq_samples=C1.slq_samples, slq_m=C1.slq_m,
        pcg_tol=C1.pcg_tol, verbose=False, return_diagnostics=True,
        slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    ctx = _oracle_ctx(K, y, X, atoms, probes)
    po, _, cur = oreml.fit(ctx, minq_iter=C1.minq_iter)
    h2 = oreml.heritability(param, 1, atoms)
    h2_ref = oreml.heritability(po, 1, atoms)
    assert abs(h2 - h2_ref) < 1e-3, (h2, h2_ref)
    assert 0.3 < h2 < 0.7
    assert abs(diag["loglik"] - cur["ll"]) <= 1e-4 * abs(cur["ll"])
    # Objective and log-determinant at the GPU's own estimate.
    at = oreml.evaluate(ctx, np.asarray(param, np.float64))
    assert abs(diag["loglik"] - at["ll"]) <= 1e-4 * abs(at["ll"]), (diag["loglik"], at["ll"])
    assert abs(diag["logdet"] - at["logdet"]) <= 1e-4 * abs(at["logdet"]), (diag["logdet"],
                                                                           at["logdet"])


def test_c1_scoring_fit_with_65_column_block(cuda, c1):
    """optimizer="smile_scoring": the phenotype and 64 Rademacher trace probes
    ride in the main block PCG as one right-hand-side block ([X | y | 64
    probes], the 65-column form plus the covariates); traces come from the
    probe columns of the solves (reml.py:608-682, :1422-1427, :1584-1595)."""
    st, K, y, X, atoms = c1
    n = y.size
    iters = 8
    slq = np.random.default_rng(C1.seed).choice([-1.0, 1.0], size=(n, C1.slq_samples))
    tp = np.random.default_rng(C1.seed + 1).choice([-1.0, 1.0], size=(n, 64))
    param, hist, diag = greml.fit_reml(
        y, [lambda V: st.kv(V)], [st.diag()], X, n_rand_vec=64, maxiter=1000, minq_iter=iters,
        slq_samples=C1.slq_samples, slq_m=C1.slq_m, pcg_tol=C1.pcg_tol, verbose=False,
        return_diagnostics=True, optimizer="smile_scoring",
        slq_probes=torch.as_tensor(slq, dtype=torch.float32),
        trace_probes=torch.as_tensor(tp, dtype=torch.float32))
    ctx = _oracle_ctx(K, y, X, atoms, slq, trace_probes=tp)
    po, ho, cur = oreml.fit_scoring(ctx, minq_iter=iters)
    assert len(hist) == len(ho)
    assert [h["slq_taylor"] for h in hist] == [h["taylor"] for h in ho]
    h2 = oreml.heritability(param, 1, atoms)
    h2_ref = oreml.heritability(po, 1, atoms)
    assert abs(h2 - h2_ref) < 1e-3, (h2, h2_ref)
    assert abs(diag["loglik"] - cur["ll"]) <= 1e-4 * abs(cur["ll"])
    trK, trR = oreml.hutchinson_traces(ctx, cur["sol"])
    np.testing.assert_allclose(diag["trace_K"], trK, rtol=1e-4)
    np.testing.assert_allclose(diag["trace_R"], trR, rtol=1e-4)
    assert abs(diag["logdet"] - cur["logdet"]) <= 1e-4 * abs(cur["logdet"])
