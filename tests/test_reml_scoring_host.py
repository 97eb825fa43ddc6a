"""The scoring optimizer's pieces (reml.py:608-682, :821-857, :1700-1880 of the
reference) on CPU, with dense kernels and pcg_solve replaced by an exact
solve.  A Taylor evaluation takes the given log-determinant and forms its
score from Hutchinson traces of the projected probes; the traces of the
next Taylor expansion come from the probe columns of the solves; the driver
takes one trial per iteration, accepts downhill steps, and expands the
log-determinant when the relative step is below the threshold."""
import numpy as np
import pytest
import torch

from coherit_gb300 import reml


@pytest.fixture(autouse=True)
def _exact_solves(monkeypatch):
    def solve(Hv, B, M=None, tol=1e-2, maxiter=200, X0=None, check_every=2):
        B2 = torch.as_tensor(B).float()
        vec = B2.ndim == 1
        B2 = B2[:, None] if vec else B2
        H = torch.as_tensor(Hv(torch.eye(B2.shape[0]))).double()
        X = torch.linalg.solve(0.5 * (H + H.T), B2.double()).float()
        R = B2.double() - torch.as_tensor(Hv(X)).double()
        rel = torch.max(R.norm(dim=0) / B2.double().norm(dim=0).clamp_min(1e-300))
        return (X[:, 0] if vec else X), rel, 1

    monkeypatch.setattr(reml, "pcg_solve", solve)


def _problem(n=60, R=24, residual=False):
    rng = np.random.default_rng(31)
    Ks = []
    for w in (17, 29):
        A = rng.normal(size=(n, w))
        Ks.append(A @ A.T / w)
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = rng.normal(size=n)
    Z = rng.choice([-1.0, 1.0], size=(n, R))
    Rd = np.stack([np.ones(n), np.linspace(.5, 1.5, n)]) if residual else None
    return Ks, X, y, Z, Rd


def _context(Ks, X, y, Z, Rd):
    n, R = Z.shape
    Kt = torch.as_tensor(np.stack(Ks), dtype=torch.float32)
    ops = tuple(lambda v, k=k: k @ v for k in Kt)
    Zt = torch.as_tensor(Z, dtype=torch.float32)
    rhs = torch.column_stack([torch.as_tensor(X, dtype=torch.float32),
                              torch.as_tensor(y, dtype=torch.float32), Zt])
    return reml.REMLContext(
        n=n, G=len(Ks), E=1 if Rd is None else Rd.shape[0], K_mvs=ops, weighted_hv=None,
        stacked_kv=None, diag_stack=torch.diagonal(Kt, dim1=1, dim2=2),
        residual_diag_stack=None if Rd is None else torch.as_tensor(Rd, dtype=torch.float32),
        xmat=torch.as_tensor(X, dtype=torch.float32), y=torch.as_tensor(y, dtype=torch.float32),
        rhs_const=rhs, y_col=X.shape[1], rand_stop=rhs.shape[1], n_XyZ_cols=rhs.shape[1],
        R_rand=R, kvrand_stack=torch.stack([op(Zt) for op in ops]), precond_conf=None)


def _dense(theta, Ks, X, Rd):
    n = X.shape[0]
    G = len(Ks)
    res = [np.eye(n)] if Rd is None else [np.diag(r) for r in Rd]
    H = sum(t * K for t, K in zip(theta[:G], Ks)) + sum(t * Rm for t, Rm in zip(theta[G:], res))
    Hi = np.linalg.inv(H)
    HX = Hi @ X
    A = X.T @ HX
    P = Hi - HX @ np.linalg.solve(A, HX.T)
    return Hi, P, Ks + res, np.linalg.slogdet(A)[1]


@pytest.mark.parametrize("residual", [False, True])
def test_taylor_evaluation_uses_hutchinson_score(residual):
    Ks, X, y, Z, Rd = _problem(residual=residual)
    ctx = _context(Ks, X, y, Z, Rd)
    theta = np.array([0.4, 0.3, 0.5] + ([0.2] if residual else []))
    taylor = torch.tensor(7.25, dtype=torch.float64)
    out = reml._eval_once(ctx, theta, torch.zeros_like(ctx.rhs_const), key_slq=3, minq_tol=1e-6,
                          maxiter=100, precond_eps=1e-7, slq_samples=4, slq_m=8,
                          taylor_logdet=taylor, compute_traces=False)
    ll, grad, FI = out[0], out[1], out[2]
    Hi, P, mats, logdet_x = _dense(theta, Ks, X, Rd)
    n, R = Z.shape
    Py = P @ y
    q = np.array([Py @ M @ Py for M in mats])
    tr = np.array([np.sum((P @ Z) * (M @ Z)) / R for M in mats])
    np.testing.assert_allclose(grad, 0.5 * (q - tr) / n, rtol=2e-4, atol=1e-6)
    assert ll == pytest.approx(-0.5 * (y @ Py + 7.25 + logdet_x) / n, rel=1e-5)
    assert out[8] is taylor or float(out[8]) == 7.25
    assert FI.mat.shape == (len(theta), len(theta))


@pytest.mark.parametrize("residual", [False, True])
def test_traces_for_the_taylor_expansion_come_from_the_probe_solves(residual):
    Ks, X, y, Z, Rd = _problem(residual=residual)
    ctx = _context(Ks, X, y, Z, Rd)
    theta = np.array([0.4, 0.3, 0.5] + ([0.2] if residual else []))
    Hi, _, mats, _ = _dense(theta, Ks, X, Rd)
    sol = torch.as_tensor(Hi @ ctx.rhs_const.double().numpy(), dtype=torch.float32)
    trR, trK = reml._compute_traces_from_pcg(sol, ctx)
    R = Z.shape[1]
    HZ = Hi @ Z
    G = len(Ks)
    np.testing.assert_allclose(trK.numpy(), [np.sum(HZ * (K @ Z)) / R for K in Ks], rtol=1e-5)
    np.testing.assert_allclose(trR.numpy(), [np.sum(HZ * (M @ Z)) / R for M in mats[G:]],
                               rtol=1e-5)


def test_scoring_driver_takes_single_trials_and_expands_small_steps():
    Ks, X, y, Z, _ = _problem(n=80, R=32)
    Kt = [torch.as_tensor(K, dtype=torch.float32) for K in Ks]
    probes = np.random.default_rng(5).choice([-1.0, 1.0], size=(80, 12))
    param, hist, diag = reml.fit_reml(
        y.astype(np.float32), tuple(lambda v, k=k: k @ v for k in Kt),
        [torch.diagonal(k) for k in Kt], X, n_rand_vec=32, maxiter=300, minq_iter=12,
        slq_samples=12, slq_m=10, slq_mode="raw", pcg_tol=1e-5, verbose=False,
        return_diagnostics=True, device="cpu", optimizer="smile_scoring",
        slq_probes=torch.as_tensor(probes, dtype=torch.float32),
        trace_probes=torch.as_tensor(Z, dtype=torch.float32), taylor_threshold=0.05,
        scoring_step_tol=1e-4)
    assert all(h["line_search_trials"] == 1 and h["accepted"] for h in hist)
    assert all(h["step_alpha"] == 1.0 for h in hist)
    for h in hist:
        if h["slq_taylor"]:
            assert h["max_rel_dp"] < 0.05
    assert hist[-1]["stop_reason"] in ("scoring_step", "max_iter")
    if hist[-1]["stop_reason"] == "scoring_step":
        assert hist[-1]["max_rel_dp"] < 1e-4
    assert np.all(np.isfinite(param)) and np.isfinite(diag["loglik"])


def test_taylor_logdet_is_the_first_order_expansion(monkeypatch):
    """logdet(theta + d) ~ logdet(theta) + sum_i d_i tr(H^-1 M_i), the traces
    taken at the last full evaluation (reml.py:1800-1829)."""
    Ks, X, y, Z, _ = _problem(n=80, R=32)
    Kt = [torch.as_tensor(K, dtype=torch.float32) for K in Ks]
    calls = []
    original = reml._eval_once

    def recording(ctx, pvec, *a, taylor_logdet=None, **kw):
        out = original(ctx, pvec, *a, taylor_logdet=taylor_logdet, **kw)
        calls.append((np.array(pvec, np.float64), None if taylor_logdet is None
                      else float(taylor_logdet), float(out[8])))
        return out

    monkeypatch.setattr(reml, "_eval_once", recording)
    probes = np.random.default_rng(5).choice([-1.0, 1.0], size=(80, 12))
    reml.fit_reml(y.astype(np.float32), tuple(lambda v, k=k: k @ v for k in Kt),
                  [torch.diagonal(k) for k in Kt], X, n_rand_vec=32, maxiter=300, minq_iter=12,
                  slq_samples=12, slq_m=10, slq_mode="raw", pcg_tol=1e-5, verbose=False,
                  device="cpu", optimizer="smile_scoring",
                  slq_probes=torch.as_tensor(probes, dtype=torch.float32),
                  trace_probes=torch.as_tensor(Z, dtype=torch.float32), taylor_threshold=0.05)
    R = Z.shape[1]
    expansions = 0
    anchor_theta, anchor_logdet = calls[0][0], calls[0][2]
    for theta, taylor, logdet in calls[1:]:
        if taylor is not None:
            Hi, _, mats, _ = _dense(anchor_theta, Ks, X, None)
            tr = np.array([np.sum((Hi @ Z) * (M @ Z)) / R for M in mats])
            expected = anchor_logdet + (theta - anchor_theta) @ tr
            assert taylor == pytest.approx(expected, rel=1e-5, abs=1e-6)
            expansions += 1
        anchor_theta, anchor_logdet = theta, logdet     # every scoring step is accepted
    assert expansions >= 1
