"""Continuous-batching REML server on the GPU operator.

A fit served in a mix of concurrent requests must give the result of the
same fit run alone: |delta h2| < 1e-4 and log-likelihood within 1e-5
relative (the batched launch changes only the padding of the right-hand-side
block and the order of FP64 atomic additions).  A request over a sample
subset must match a fit on a streamer built on that subset, the way the
reference rebuilds per-sample-set statistics (geno_stream.py:1230-1247).
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import synth
from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
from coherit_gb300.reml import fit_reml
from coherit_gb300.serving import REMLServer

pytestmark = pytest.mark.gpu

N, M, SEED = 1500, 4000, 31
KW = dict(n_rand_vec=30, maxiter=500, minq_iter=20, slq_samples=30, slq_m=30, pcg_tol=1e-5,
          verbose=False)


def _h2(param, diag):
    gen = float(param[0] * diag["genetic_trace_atoms"][0])
    res = float(param[1] * diag["residual_trace_atoms"][0])
    return gen / (gen + res)


def _alone(st, y, X):
    param, _, d = fit_reml(y, [lambda V: st.kv(V)], [st.diag()], X, return_diagnostics=True,
                           device=st.dev, **KW)
    return _h2(param, d), float(d["loglik"])


@pytest.fixture(scope="module")
def problem(cuda):
    st = GenoBlockStreamer(SyntheticSource(N, M, seed=SEED), precision="bf16x3")
    phen = [synth.phenotype(SEED, N, M, h2=h, n_causal=100, n_covar=2, pheno_seed=100 + i)[:2]
            for i, h in enumerate([0.2, 0.5, 0.7, 0.4])]
    mask = np.random.default_rng(3).random(N) < 0.7
    yield st, phen, mask
    st.close()


def test_served_mix_matches_fits_alone(problem):
    st, phen, mask = problem
    sub = GenoBlockStreamer(SyntheticSource(N, M, seed=SEED), precision="bf16x3",
                            sample_mask=mask)
    reqs = [(phen[0][0], phen[0][1], None), (phen[1][0], phen[1][1], None),
            (phen[2][0][mask], phen[2][1][mask], mask), (phen[3][0][mask], phen[3][1][mask], mask)]
    expect = [_alone(st, *phen[0]), _alone(st, *phen[1]),
              _alone(sub, phen[2][0][mask], phen[2][1][mask]),
              _alone(sub, phen[3][0][mask], phen[3][1][mask])]
    sub.close()
    with REMLServer(st, max_active=4, batch_window_s=0.01, fit_kwargs=KW) as srv:
        got = srv.map(reqs)
        stats = srv.stats()
    assert stats["completed"] == 4
    # Fits ran together: launches carried more than one request on average.
    assert stats["mean_requests_per_launch"] > 1.5
    for r, (h2, ll) in zip(got, expect):
        assert abs(r.heritability - h2) < 1e-4, (r.heritability, h2)
        assert abs(r.loglik - ll) <= 1e-5 * abs(ll), (r.loglik, ll)
    assert got[2].n_samples == int(mask.sum())


def test_admission_queues_beyond_max_active(problem):
    st, phen, _ = problem
    kw = dict(KW, minq_iter=3)
    with REMLServer(st, max_active=2, fit_kwargs=kw) as srv:
        futs = [srv.submit(phen[i % 4][0], phen[i % 4][1]) for i in range(5)]
        res = [f.result(timeout=600) for f in futs]
        stats = srv.stats()
    assert [r.request_id for r in res] == list(range(5))
    assert stats["completed"] == 5 and stats["p99_s"] >= stats["p50_s"] > 0
    # Requests 0 and 4 carry the same phenotype: same result whatever ran beside them.
    assert abs(res[0].heritability - res[4].heritability) < 1e-4
    starts = sorted(r.start for r in res)
    finishes = sorted(r.finish for r in res)
    # At most two in flight: the third start comes after the first finish.
    assert starts[2] >= finishes[0]


def test_bad_requests_fail_alone(problem):
    st, phen, mask = problem
    with REMLServer(st, max_active=2, fit_kwargs=dict(KW, minq_iter=2)) as srv:
        with pytest.raises(ValueError):
            srv.submit(phen[0][0][:10])
        with pytest.raises(ValueError):
            srv.submit(phen[0][0], sample_mask=mask)
        bad = srv.submit(np.full(N, np.nan, dtype=np.float32))
        good = srv.submit(phen[1][0], phen[1][1])
        with pytest.raises(Exception):
            bad.result(timeout=600)
        assert np.isfinite(good.result(timeout=600).heritability)
    with pytest.raises(RuntimeError):
        srv.submit(phen[0][0])


def test_projected_core_preconditioner_per_request(problem):
    """Served fits with a per-request projected-core preconditioner (one basis
    for the full cohort, one per subset request, reml_model.py:863-960) give
    the fits without it: the preconditioner changes how PCG converges, not
    the solutions (|delta h2| < 5e-4, log-likelihood within 1e-4 relative at
    PCG tolerance 1e-5)."""
    st, phen, mask = problem
    reqs = [(phen[1][0], phen[1][1], None), (phen[2][0][mask], phen[2][1][mask], mask)]
    with REMLServer(st, max_active=2, fit_kwargs=KW) as srv:
        base = srv.map(reqs)
    with REMLServer(st, max_active=2, fit_kwargs=KW, precond_rank=48) as srv:
        got = srv.map(reqs)
        conf = srv._full_precond
    assert conf is not None and conf.total_rank == 48
    U = conf.U.double()
    eye = torch.eye(48, dtype=torch.float64, device=U.device)
    assert torch.allclose(U.T @ U, eye, atol=1e-4)
    for r, b in zip(got, base):
        assert r.n_samples == b.n_samples
        assert abs(r.heritability - b.heritability) < 5e-4, (r.heritability, b.heritability)
        assert abs(r.loglik - b.loglik) <= 1e-4 * abs(b.loglik), (r.loglik, b.loglik)
