"""REML fits on the GPU operator versus the FP64 oracle (same genotypes, same probes).

Tolerances: |delta h2| < 1e-3, log-likelihood and log-determinant within 1e-4
relative, score/AI entries within 1e-4 relative of their scale.
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import reml as greml
from coherit_gb300 import synth
from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter
from oracle import geno as og
from oracle import reml as oreml
from oracle import slq as oslq

pytestmark = pytest.mark.gpu


def _problem(n, m, seed, comps=None, miss=0.0, h2=0.5, n_causal=200, n_covar=2):
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=seed, missing_rate=miss),
                           component_block_sizes=comps, precision="bf16x3")
    codes = og.synth_codes(seed, n, np.arange(m), missing_q24=synth.missing_rate_q24(miss))
    y, X, _, _ = synth.phenotype(seed, n, m, h2=h2, n_causal=n_causal,
                                 missing_q24=synth.missing_rate_q24(miss), n_covar=n_covar)
    return st, codes, y, X


def _dense_kernels(st, codes, comps):
    mean, inv = st._means_host, st._inv_sds_host
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)[None, :]
    Ks = []
    pos = 0
    for g, size in enumerate(comps):
        Zg = Z[:, pos:pos + size]
        Ks.append(Zg @ Zg.T / float(st._component_eff_m_host[g]))
        pos += size
    return Ks


def test_single_grm_fit_matches_oracle(cuda):
    n, m = 1000, 5000
    st, codes, y, X = _problem(n, m, seed=21)
    (K,) = _dense_kernels(st, codes, [m])
    probes = np.random.default_rng(5).choice([-1.0, 1.0], size=(n, 30))
    kw = dict(n_rand_vec=30, maxiter=500, minq_iter=20, slq_samples=30, slq_m=30, pcg_tol=1e-6,
              verbose=False, return_diagnostics=True)
    param, hist, diag = greml.fit_reml(
        y, [lambda V: st.kv(V)], [st.diag()], X, slq_probes=torch.as_tensor(probes, dtype=torch.float32),
        **kw)
    yo, _, _ = oreml.standardize(y)
    cache = oslq.affine_cache(lambda v: K @ v, n, probes, 30)
    ctx = oreml.Context(yo, [lambda v: K @ v], X, diag_atoms=[float(st._mean_diag_atom_host)],
                        affine_cache=cache, pcg_tol=1e-6, maxiter=500)
    po, ho, cur = oreml.fit(ctx, minq_iter=20)
    atoms = [float(st._mean_diag_atom_host)]
    h2_gpu = oreml.heritability(param, 1, atoms)
    h2_ref = oreml.heritability(po, 1, atoms)
    assert abs(h2_gpu - h2_ref) < 1e-3, (h2_gpu, h2_ref)
    assert abs(diag["loglik"] - cur["ll"]) <= 1e-4 * abs(cur["ll"])
    assert 0.2 < h2_gpu < 0.8


def test_eval_once_score_and_ai_match_oracle(cuda):
    n, m = 700, 3000
    comps = [1000, 2000]
    st, codes, y, X = _problem(n, m, seed=23, comps=comps, miss=0.01)
    Ks = _dense_kernels(st, codes, comps)
    probes = np.random.default_rng(6).choice([-1.0, 1.0], size=(n, 8))
    yo, _, _ = oreml.standardize(y)
    theta = np.asarray([0.3, 0.25, 0.5])
    ctx_o = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X,
                          diag_atoms=st._component_mean_diag_atoms_host, slq_probes=probes,
                          slq_m=12, pcg_tol=1e-6, maxiter=500)
    ref = oreml.evaluate(ctx_o, theta)
    dev = cuda
    ytd = torch.as_tensor(yo, device=dev)
    Xd = torch.as_tensor(X, device=dev)
    rhs = torch.cat([Xd, ytd[:, None]], dim=1).contiguous()
    ctx = greml.REMLContext(
        n=n, G=2, E=1, K_mvs=tuple((lambda V, g=g: st.component_kv(V, g)) for g in range(2)),
        weighted_hv=lambda tg, te, V: st.weighted_component_hv(tg, te, V),
        stacked_kv=lambda V: st.stacked_component_kv(V), diag_stack=None,
        residual_diag_stack=None, xmat=Xd, y=ytd, rhs_const=rhs, y_col=X.shape[1],
        rand_stop=X.shape[1] + 1, n_XyZ_cols=X.shape[1] + 1, R_rand=0, kvrand_stack=None,
        precond_conf=None, diag_atoms=st._component_mean_diag_atoms_host.astype(np.float64),
        slq_probes=torch.as_tensor(probes, dtype=torch.float32, device=dev))
    out = greml._eval_once(ctx, theta, None, key_slq=0, minq_tol=1e-6, maxiter=500,
                           precond_eps=1e-6, slq_samples=8, slq_m=12)
    ll, grad, FI = out[0], out[1], out[2]
    assert abs(ll - ref["ll"]) <= 1e-4 * abs(ref["ll"])
    np.testing.assert_allclose(grad, ref["grad"], rtol=1e-3, atol=1e-4 * np.max(np.abs(ref["grad"])))
    np.testing.assert_allclose(FI.mat, ref["ai"], rtol=1e-3, atol=1e-5)


def test_fitter_with_preconditioner_two_components(cuda):
    n, m = 800, 4000
    comps = [1500, 2500]
    st, codes, y, X = _problem(n, m, seed=29, comps=comps, h2=0.4)
    Ks = _dense_kernels(st, codes, comps)
    cfg = FitConfig(slq_samples=16, slq_m=16, precond_rank=64, reml_pcg_tol=1e-5, minq_iter=15,
                    max_pcg_iters=500, slq_mode="raw")
    probes = np.random.default_rng(9).choice([-1.0, 1.0], size=(n, 16))
    res = InfinitesimalREMLFitter(cfg, [st]).fit_infinitesimal(
        y, X, slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    yo, _, _ = oreml.standardize(y)
    ctx_o = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X,
                          diag_atoms=st._component_mean_diag_atoms_host, slq_probes=probes,
                          slq_m=16, pcg_tol=1e-5, maxiter=500)
    po, _, _ = oreml.fit(ctx_o, minq_iter=15)
    atoms = st._component_mean_diag_atoms_host.astype(np.float64)
    h2_ref = oreml.heritability(po, 2, atoms)
    assert abs(res.heritability - h2_ref) < 1e-3, (res.heritability, h2_ref)


def test_slq_probe_batching_does_not_change_value_or_gradient(cuda):
    """The SLQ workspace decides how many probes share one operator
    application (slq.py:24-41); each probe's Lanczos recurrence is
    independent, so one probe per batch and all probes in one batch give
    the same log-determinant and gradient up to the FP32 rounding of the
    products at another block width (1e-5 relative)."""
    from coherit_gb300 import slq

    n, p, m = 400, 8, 12
    rng = np.random.default_rng(2)
    A = rng.standard_normal((n, n // 2))
    K = torch.as_tensor(A @ A.T / (n // 2), dtype=torch.float32, device=cuda)
    theta = np.array([0.6, 0.4])

    def Hv(v):
        return float(theta[0]) * (K @ v) + float(theta[1]) * v

    def pullback(left, right):
        kl = K @ left
        res = float(theta[0]) * kl + float(theta[1]) * left
        scores = torch.stack([torch.sum(right.double() * kl.double()),
                              torch.sum(right.double() * left.double())])
        return res, scores

    probes = torch.as_tensor(rng.choice([-1.0, 1.0], size=(n, p)), dtype=torch.float32,
                             device=cuda)
    per_probe = 4 * n * (8 * (m + 1) + 32)
    out = []
    for ws in (per_probe, 64 * per_probe):
        assert slq.workspace_layout(n, p, m, ws)["batch_width"] in (1, p)
        v, g = slq.logdet_value_and_grad(Hv, pullback, n, 0, nsamples=p, m=m,
                                         workspace_bytes=ws, probes=probes)
        out.append((float(v), g.cpu().numpy()))
    assert abs(out[0][0] - out[1][0]) <= 1e-5 * abs(out[1][0])
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-5, atol=1e-8)
