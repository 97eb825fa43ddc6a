"""The reference's score-consistency checks on the package's _eval_once (CPU).

tests/test_multi_slq_score_consistency.py:140-216 and
tests/test_affine_slq_score_consistency.py:20-146 of the reference: the
returned score is the derivative of the returned REML objective (central
finite differences), the strict gate returns the same value and either the
same score or none, and the AI direction is an ascent direction.  The multi-
component case runs with covariates, two residual components, a zero
genetic component and SLQ whitening by a frozen projected-core reference.
Dense FP32 kernels on CPU; pcg_solve is replaced by an exact solve.
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import precond, reml

CPU = torch.device("cpu")


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


def _regular_kernels():
    # tests/test_multi_slq_score_consistency.py:19-35 of the reference ("regular")
    rng = np.random.default_rng(904)
    n = 24
    kernels = []
    for width in (13, 21, 37):
        raw = rng.normal(size=(n, width))
        kernels.append(raw @ raw.T / width)
    return np.stack(kernels), np.array([.21, .16, .28, .57])


@pytest.mark.parametrize("with_covar,with_reference,multiple_residual,zero_component", [
    (False, False, False, False),
    (True, False, False, False),
    (True, True, False, False),
    (True, True, True, False),
    (True, True, False, True),
])
def test_integrated_reml_score_matches_its_objective(with_covar, with_reference,
                                                     multiple_residual, zero_component):
    matrices, theta = _regular_kernels()
    n = matrices.shape[1]
    rng = np.random.default_rng(91)
    kernels = torch.as_tensor(matrices, dtype=torch.float32)
    operators = tuple(lambda b, k=k: k @ b for k in kernels)
    residual = None
    if multiple_residual:
        residual = torch.as_tensor(np.stack([np.ones(n), np.linspace(.3, 1.5, n)]),
                                   dtype=torch.float32)
        theta = np.r_[theta, .16]
    if zero_component:
        theta[0] = 0
    covar = (torch.as_tensor(np.column_stack([np.ones(n), rng.normal(size=n)]),
                             dtype=torch.float32) if with_covar else None)
    y = torch.as_tensor(rng.normal(size=n), dtype=torch.float32)
    probes = torch.as_tensor(rng.choice([-1., 1.], size=(n, 4)), dtype=torch.float32)
    cols = 0 if covar is None else covar.shape[1]
    rhs = torch.column_stack([y, probes] if covar is None else [covar, y, probes])
    ctx = reml.REMLContext(
        n=n, G=3, E=2 if multiple_residual else 1, K_mvs=operators, weighted_hv=None,
        stacked_kv=None, diag_stack=torch.diagonal(kernels, dim1=1, dim2=2),
        residual_diag_stack=residual, xmat=covar, y=y, rhs_const=rhs, y_col=cols,
        rand_stop=rhs.shape[1], n_XyZ_cols=rhs.shape[1], R_rand=4,
        kvrand_stack=torch.stack([op(probes) for op in operators]), precond_conf=None)
    if with_reference:
        basis = torch.as_tensor(np.linalg.qr(rng.normal(size=(n, 4)))[0], dtype=torch.float32)
        eigvals = torch.tensor([1.1, 1.3, 1.7, 2.1])
        ctx.slq_reference_runtime = precond.ProjectedCoreRuntime(
            U=basis, total_rank=4, d=torch.tensor(.9), d_inv=torch.tensor(1 / .9),
            chol=torch.diag(torch.sqrt(eigvals)), eigvals=eigvals, eigvecs=torch.eye(4))

    def evaluate(t, **kw):
        return reml._eval_once(ctx, np.asarray(t, np.float64), torch.zeros_like(rhs),
                               key_slq=83, minq_tol=2e-6, maxiter=200, precond_eps=1e-7,
                               slq_samples=4, slq_m=10, slq_mode="projected_core_residual",
                               compute_traces=False, **kw)

    value, gradient, information, *_ = evaluate(theta)
    accepted = evaluate(theta, min_loglik=value)
    rejected = evaluate(theta, min_loglik=value + .1)
    assert accepted[0] == value and rejected[0] == value
    np.testing.assert_array_equal(accepted[1], gradient)
    np.testing.assert_array_equal(accepted[2].mat, information.mat)
    assert rejected[1] is None and rejected[2] is None
    fd = []
    for k in range(len(theta)):
        delta = np.eye(len(theta))[k] * .001
        if theta[k] == 0:
            fd.append((evaluate(theta + delta)[0] - value) / .001)
        else:
            fd.append((evaluate(theta + delta)[0] - evaluate(theta - delta)[0]) / .002)
    np.testing.assert_allclose(gradient, fd, atol=6e-4, rtol=5e-3)
    if not zero_component:
        direction = np.linalg.solve(information.mat + np.eye(len(theta)) * information.ridge,
                                    gradient)
        assert float(gradient @ direction) > 0
        step = min(.002, .05 * float(np.min(theta / np.maximum(abs(direction), 1e-9))))
        assert evaluate(theta + step * direction)[0] > value


def _affine_context(with_fixed_effects):
    # tests/test_affine_slq_score_consistency.py:24-77 of the reference
    rng = np.random.default_rng(20260723)
    n = 10
    raw = rng.normal(size=(n, 14))
    kernel = torch.as_tensor(raw @ raw.T / raw.shape[1] + 0.08 * np.eye(n), dtype=torch.float32)
    y = torch.as_tensor(rng.normal(size=n), dtype=torch.float32)
    xmat = (torch.as_tensor(np.column_stack([np.ones(n), rng.normal(size=n)]),
                            dtype=torch.float32) if with_fixed_effects else None)
    probes = torch.as_tensor(rng.choice([-1.0, 1.0], size=(n, 6)), dtype=torch.float32)
    x_cols = 0 if xmat is None else xmat.shape[1]
    rhs = torch.cat(([xmat] if xmat is not None else []) + [y[:, None], probes], dim=1)
    K = (lambda v: kernel @ v,)
    cache = reml._build_affine_slq_cache(K[0], n, 991, nsamples=5, m=n, device=CPU)
    return reml.REMLContext(
        n=n, G=1, E=1, K_mvs=K, weighted_hv=None, stacked_kv=None,
        diag_stack=torch.diagonal(kernel)[None, :], residual_diag_stack=None, xmat=xmat, y=y,
        rhs_const=rhs, y_col=x_cols, rand_stop=x_cols + 1 + 6, n_XyZ_cols=rhs.shape[1],
        R_rand=6, kvrand_stack=(kernel @ probes)[None], precond_conf=None,
        affine_slq_cache=cache)


def _affine_eval(ctx, theta):
    return reml._eval_once(ctx, np.asarray(theta, np.float64), torch.zeros_like(ctx.rhs_const),
                           warm_ai=torch.zeros((ctx.n, 2)), key_slq=991, minq_tol=2e-6,
                           maxiter=100, precond_eps=1e-7, slq_samples=5, slq_m=ctx.n,
                           slq_mode="raw", compute_traces=False)


@pytest.mark.parametrize("with_fixed_effects", [False, True])
def test_affine_score_matches_finite_difference(with_fixed_effects):
    ctx = _affine_context(with_fixed_effects)
    theta = np.asarray([0.37, 0.74])
    ll, grad, *_ = _affine_eval(ctx, theta)
    assert np.isfinite(ll)
    eps = 2e-3
    fd = [(_affine_eval(ctx, theta + eps * e)[0] - _affine_eval(ctx, theta - eps * e)[0])
          / (2 * eps) for e in np.eye(2)]
    np.testing.assert_allclose(grad, fd, atol=7e-4, rtol=7e-3)


def test_affine_ai_direction_is_an_ascent_direction():
    ctx = _affine_context(True)
    theta = np.asarray([0.22, 0.91])
    ll, grad, ai, *_ = _affine_eval(ctx, theta)
    direction = np.linalg.solve(0.5 * (ai.mat + ai.mat.T) + ai.ridge * np.eye(2), grad)
    assert float(grad @ direction) > 0
    imp = [_affine_eval(ctx, theta + a * direction)[0] - ll
           for a in (0.25, 0.125, 0.0625, 0.03125, 0.015625) if np.all(theta + a * direction > 0)]
    assert imp and max(imp) > 0
