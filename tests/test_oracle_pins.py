"""Pin the CPU oracle to the known-answer checks of the reference's own tests.

Each test restates one check of the reference suite (file:line given) and
runs it against the oracle restatement.  The package runs the same checks:
the PCG ones on the GPU (test_gpu_pcg.py), the SLQ, affine-SLQ and Fisher-step
ones on CPU tensors (test_reml_host.py), since that code reaches the device
only through the operator callable.
"""
import numpy as np
import pytest

from oracle import pcg as opcg


def _true_relative(hv, x, b):
    residual = np.asarray(b - hv(x), dtype=np.float64)
    rhs = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(rhs, axis=0)
    return float(np.max(np.linalg.norm(residual, axis=0) / np.where(den > 0, den, 1)))


# tests/test_pcg_stability.py:26-48
@pytest.mark.parametrize("check_every", [1, 2, 5])
@pytest.mark.parametrize("preconditioned", [False, True])
def test_pcg_diagonal_zero_and_extreme_scales(check_every, preconditioned):
    scales = np.asarray([0, 1e-30, 1e-8, 1, 1e30], dtype=np.float32)
    b = np.arange(1, 17, dtype=np.float32)[:, None] * scales
    calls = []

    def hv(v):
        calls.append(None)
        return 2 * v

    pre = (lambda v: v / 2) if preconditioned else None
    x, rel, it = opcg.pcg_solve(hv, b, M=pre, tol=1e-6, maxiter=20, check_every=check_every)
    assert len(calls) == it + 2
    np.testing.assert_allclose(x[:, 1:] / scales[1:],
                               np.broadcast_to(np.arange(1, 17)[:, None] / 2, (16, 4)), rtol=1e-6)
    np.testing.assert_array_equal(x[:, 0], 0)
    assert rel == pytest.approx(_true_relative(hv, x, b), abs=1e-8)
    assert rel <= 1e-6
    assert it <= check_every


# tests/test_pcg_stability.py:51-68
@pytest.mark.parametrize("preconditioned", [False, True])
def test_pcg_spd_dense_with_warm_start(preconditioned):
    rng = np.random.default_rng(237)
    root = rng.normal(size=(24, 24))
    h = (root @ root.T / 24 + np.eye(24)).astype(np.float32)
    rhs = rng.normal(size=(24, 3)).astype(np.float32)
    scales = np.asarray([1e-20, 1, 1e20], dtype=np.float32)
    b = rhs * scales
    x0 = 0.1 * b
    hv = lambda v: (h.astype(np.float64) @ v.astype(np.float64)).astype(np.float32)
    pre = (lambda v: v / np.diag(h)[:, None]) if preconditioned else None
    x, rel, _ = opcg.pcg_solve(hv, b, M=pre, X0=x0, tol=1e-6, maxiter=100)
    expected = np.linalg.solve(h.astype(np.float64), rhs)
    np.testing.assert_allclose(x / scales, expected, atol=2e-6, rtol=2e-5)
    assert rel <= 1e-6
    assert rel == pytest.approx(_true_relative(hv, x, b), rel=2e-6, abs=1e-12)


# tests/test_pcg_stability.py:71-80
def test_pcg_converged_warm_start_preserved():
    d = np.arange(1, 9, dtype=np.float32)[:, None]
    hv = lambda v: d * v
    b = (np.arange(8, dtype=np.float32) * 1e-20)[:, None]
    x0 = b / d
    x, rel, it = opcg.pcg_solve(hv, b, X0=x0, tol=1e-6)
    np.testing.assert_array_equal(x, x0)
    assert it == 0


# tests/test_pcg_stability.py:83-87
def test_pcg_zero_rhs_ignores_warm_start():
    b = np.asarray([[0, 1], [0, -2], [0, 3]], dtype=np.float32)
    x, rel, _ = opcg.pcg_solve(lambda v: v, b, X0=np.ones_like(b), tol=1e-6)
    np.testing.assert_array_equal(x, b)
    assert rel == 0


# tests/test_pcg_stability.py:90-99
@pytest.mark.parametrize("maxiter", [1, 314])
def test_pcg_reports_true_residual_at_budget(maxiter):
    rng = np.random.default_rng(12)
    basis = np.linalg.qr(rng.normal(size=(60, 60)))[0]
    h = ((basis * np.geomspace(1, 1e4, 60)) @ basis.T).astype(np.float32)
    b = rng.normal(size=(60, 2)).astype(np.float32)
    hv = lambda v: (h.astype(np.float64) @ v.astype(np.float64)).astype(np.float32)
    x, rel, it = opcg.pcg_solve(hv, b, tol=1e-5, maxiter=maxiter)
    assert it <= maxiter
    assert rel == pytest.approx(_true_relative(hv, x, b), rel=2e-6, abs=1e-10)


# tests/test_pcg_stability.py:102-133
@pytest.mark.parametrize("maxiter", [1, 100])
def test_pcg_optimistic_recurrence_restarts(maxiter):
    calls = {"updates": 0, "operator": 0}

    def lose_once(*args):
        x, r, bd = opcg._state_update(*args)
        calls["updates"] += 1
        if calls["updates"] == 1:
            r = np.zeros_like(r)
        return x, r, bd

    d = np.linspace(1, 4, 20, dtype=np.float32)[:, None]
    b = np.ones((20, 1), np.float32)

    def hv(v):
        calls["operator"] += 1
        return d * v

    x, rel, it = opcg.pcg_solve(hv, b, tol=1e-6, maxiter=maxiter, check_every=1,
                                state_update=lose_once)
    assert rel == pytest.approx(_true_relative(hv, x, b), rel=2e-6, abs=1e-10)
    assert it <= maxiter
    if maxiter == 1:
        assert rel > 1e-6
    else:
        assert calls["operator"] > it + 2
        assert rel <= 1e-6
        np.testing.assert_allclose(x, b / d, rtol=3e-6)


# tests/test_pcg_stability.py:136-141
def test_pcg_zero_budget():
    b = np.ones((5, 2), np.float32) * 1e-20
    x, rel, it = opcg.pcg_solve(lambda v: 2 * v, b, maxiter=0)
    np.testing.assert_array_equal(x, 0)
    assert it == 0
    assert rel == pytest.approx(1)


# tests/test_pcg_stability.py:144-147
@pytest.mark.parametrize("factor", [0, -1, np.nan])
def test_pcg_invalid_operator_raises(factor):
    with pytest.raises(FloatingPointError):
        opcg.pcg_solve(lambda v: factor * v, np.ones((8, 1), np.float32), maxiter=4)


# ---------------------------------------------------------------- SLQ pins
from oracle import slq as oslq


def _slq_problem(kind):
    # tests/test_multi_slq_score_consistency.py:19-35
    rng = np.random.default_rng(904)
    n = 24
    kernels = []
    for width in (13, 21, 37):
        raw = rng.normal(size=(n, width))
        kernels.append(raw @ raw.T / width)
    if kind == "scalar":
        kernels = [np.eye(n), 2 * np.eye(n), 3 * np.eye(n)]
    elif kind == "clustered":
        kernels = [np.eye(n) + 1e-4 * k for k in kernels]
    theta = np.array([.21, .16, .28, .57])
    if kind == "zero":
        theta[:3] = 0
    elif kind == "ill_conditioned":
        theta[:] = [.8, .01, .01, .002]
    return np.stack([*kernels, np.eye(n)]), theta


_PROBES = np.random.default_rng(73).choice([-1.0, 1.0], size=(24, 4))


def _slq_oracle(directions, theta, depth, budget=64 * 1024 ** 2, value_only=False,
                eps=float(np.finfo(np.float64).eps)):
    matrix = np.einsum("k,kij->ij", theta, directions)

    def mv(v):
        return matrix @ v

    def pullback(left, right):
        products = np.einsum("kij,js->kis", directions, left)
        return np.einsum("k,kns->ns", theta, products), np.einsum("ns,kns->k", right, products)

    return oslq.logdet_value_and_grad(mv, None if value_only else pullback, 24, _PROBES,
                                      m=depth, workspace_bytes=budget, itemsize=8, eps=eps)


# tests/test_multi_slq_score_consistency.py:54-71
@pytest.mark.parametrize("kind", ["regular", "scalar", "clustered", "zero", "ill_conditioned"])
@pytest.mark.parametrize("depth", [1, 10, 30])
def test_slq_gradient_matches_finite_difference(kind, depth):
    d, t = _slq_problem(kind)
    value, grad = _slq_oracle(d, t, depth)
    delta = 1e-6 if kind == "ill_conditioned" else 2e-5
    fd = []
    for k in range(len(t)):
        off = np.eye(len(t))[k] * delta
        if t[k] == 0:
            fd.append((_slq_oracle(d, t + off, depth)[0] - value) / delta)
        else:
            fd.append((_slq_oracle(d, t + off, depth)[0] - _slq_oracle(d, t - off, depth)[0])
                      / (2 * delta))
    np.testing.assert_allclose(grad, fd, rtol=2e-3, atol=3e-3)


# tests/test_multi_slq_score_consistency.py:74-97
@pytest.mark.parametrize("kind", ["regular", "scalar", "clustered", "zero", "ill_conditioned"])
def test_slq_full_depth_equals_dense_probe_form(kind):
    d, t = _slq_problem(kind)
    eps32 = float(np.finfo(np.float32).eps)
    value, grad = _slq_oracle(d, t, 50, eps=eps32)
    matrix = np.einsum("k,kij->ij", t, d)
    vals, vecs = np.linalg.eigh(matrix)
    z = _PROBES
    log_matrix = (vecs * np.log(vals)) @ vecs.T
    expected = np.einsum("ns,nm,ms->", z, log_matrix, z) / 4
    assert np.isfinite(grad).all()
    np.testing.assert_allclose(value, expected, rtol=1e-3, atol=1e-3)
    gap = vals[:, None] - vals[None, :]
    divided = np.divide(np.log(vals[:, None]) - np.log(vals[None, :]), gap,
                        out=1 / np.broadcast_to(vals, gap.shape).copy(), where=np.abs(gap) > 1e-12)
    coeff = vecs.T @ z
    gm = vecs @ (divided * (coeff @ coeff.T / 4)) @ vecs.T
    expected_grad = np.einsum("ij,kij->k", gm, d)
    np.testing.assert_allclose(grad, expected_grad, rtol=2e-3, atol=2e-3)
    vo = _slq_oracle(d, t, 50, value_only=True, eps=eps32)
    assert vo[0] == value and vo[1] is None


# tests/test_multi_slq_score_consistency.py:100-107
def test_slq_probe_batching_invariance():
    d, t = _slq_problem("regular")
    full = _slq_oracle(d, t, 10)
    single = _slq_oracle(d, t, 10, budget=1)
    np.testing.assert_allclose(single[0], full[0], atol=1e-10)
    np.testing.assert_allclose(single[1], full[1], atol=1e-9)


# tests/test_affine_slq_score_consistency.py:149-169
def test_affine_slq_derivatives_finite_at_zero_genetic_variance():
    rng = np.random.default_rng(20260723)
    n = 10
    raw = rng.normal(size=(n, 14))
    K = raw @ raw.T / raw.shape[1] + 0.08 * np.eye(n)
    cache = oslq.affine_cache(lambda v: K @ v, n, rng.choice([-1.0, 1.0], size=(n, 5)), n)
    ld, der = oslq.affine_logdet(cache, 0.0, 1.0)
    assert np.isfinite(ld) and np.all(np.isfinite(der))
    eps = 2e-3
    fwd = (oslq.affine_logdet(cache, eps, 1.0)[0] - ld) / eps
    np.testing.assert_allclose(der[0], fwd, atol=2e-2, rtol=2e-2)
    np.testing.assert_allclose(der[1], n, atol=2e-4, rtol=2e-5)


def test_affine_slq_full_depth_equals_exact_logdet():
    rng = np.random.default_rng(5)
    n = 12
    raw = rng.normal(size=(n, 20))
    K = raw @ raw.T / 20
    z = rng.choice([-1.0, 1.0], size=(n, 6))
    cache = oslq.affine_cache(lambda v: K @ v, n, z, n)
    for tg, te in [(0.4, 0.6), (1.3, 0.2)]:
        ld, der = oslq.affine_logdet(cache, tg, te)
        H = tg * K + te * np.eye(n)
        vals, vecs = np.linalg.eigh(H)
        expected = np.einsum("ns,nm,ms->", z, (vecs * np.log(vals)) @ vecs.T, z) / 6
        np.testing.assert_allclose(ld, expected, rtol=1e-6)
        h = 1e-6
        fd_g = (oslq.affine_logdet(cache, tg + h, te)[0] - oslq.affine_logdet(cache, tg - h, te)[0]) / (2 * h)
        np.testing.assert_allclose(der[0], fd_g, rtol=1e-5)


# ---------------------------------------------------------------- REML pins
from oracle import reml as oreml


def _affine_ctx(with_fixed):
    # tests/test_affine_slq_score_consistency.py:24-77
    rng = np.random.default_rng(20260723)
    n = 10
    raw = rng.normal(size=(n, 14))
    K = raw @ raw.T / raw.shape[1] + 0.08 * np.eye(n)
    y = rng.normal(size=n)
    X = np.column_stack([np.ones(n), rng.normal(size=n)]) if with_fixed else None
    probes = rng.choice([-1.0, 1.0], size=(n, 5))
    cache = oslq.affine_cache(lambda v: K @ v, n, probes, n)
    return oreml.Context(y, [lambda v: K @ v], X, diag_atoms=[np.mean(np.diag(K))],
                         affine_cache=cache, pcg_tol=2e-6, maxiter=100)


# tests/test_affine_slq_score_consistency.py:102-125
@pytest.mark.parametrize("with_fixed", [False, True])
def test_affine_score_matches_objective_finite_difference(with_fixed):
    ctx = _affine_ctx(with_fixed)
    theta = np.asarray([0.37, 0.74])
    base = oreml.evaluate(ctx, theta)
    eps = 2e-3
    fd = []
    for c in range(2):
        off = np.zeros(2)
        off[c] = eps
        fd.append((oreml.evaluate(ctx, theta + off)["ll"] - oreml.evaluate(ctx, theta - off)["ll"])
                  / (2 * eps))
    np.testing.assert_allclose(base["grad"], fd, atol=7e-4, rtol=7e-3)


# tests/test_affine_slq_score_consistency.py:128-146
def test_affine_ai_direction_is_ascent():
    ctx = _affine_ctx(True)
    theta = np.asarray([0.22, 0.91])
    base = oreml.evaluate(ctx, theta)
    d = np.linalg.solve(base["ai"] + oreml.RIDGE * np.eye(2), base["grad"])
    assert float(base["grad"] @ d) > 0
    imp = [oreml.evaluate(ctx, theta + a * d)["ll"] - base["ll"]
           for a in (0.25, 0.125, 0.0625, 0.03125, 0.015625) if np.all(theta + a * d > 0)]
    assert imp and max(imp) > 0


# tests/test_multi_slq_score_consistency.py:140-216 (no sparse mean term, no whitening)
@pytest.mark.parametrize("with_covar", [False, True])
@pytest.mark.parametrize("multiple_residual", [False, True])
def test_multi_component_score_matches_objective(with_covar, multiple_residual):
    mats, theta = _slq_problem("regular")
    n = 24
    rng = np.random.default_rng(91)
    Ks = [(lambda v, k=k: k @ v) for k in mats[:3]]
    R = None
    if multiple_residual:
        R = np.stack([np.ones(n), np.linspace(.3, 1.5, n)])
        theta = np.r_[theta, .16]
    X = np.column_stack([np.ones(n), rng.normal(size=n)]) if with_covar else None
    y = rng.normal(size=n)
    probes = rng.choice([-1.0, 1.0], size=(n, 4))
    ctx = oreml.Context(y, Ks, X, diag_atoms=[np.mean(np.diag(k)) for k in mats[:3]],
                        slq_probes=probes, slq_m=10, pcg_tol=2e-6, maxiter=200, residual_diags=R)
    base = oreml.evaluate(ctx, theta)
    acc = oreml.evaluate(ctx, theta, min_loglik=base["ll"])
    rej = oreml.evaluate(ctx, theta, min_loglik=base["ll"] + .1)
    assert acc["ll"] == base["ll"] and rej["ll"] == base["ll"]
    np.testing.assert_array_equal(acc["grad"], base["grad"])
    assert rej["grad"] is None and rej["ai"] is None
    fd = []
    for k in range(len(theta)):
        dlt = np.eye(len(theta))[k] * .001
        fd.append((oreml.evaluate(ctx, theta + dlt)["ll"] - oreml.evaluate(ctx, theta - dlt)["ll"]) / .002)
    np.testing.assert_allclose(base["grad"], fd, atol=6e-4, rtol=5e-3)
    d = np.linalg.solve(base["ai"] + np.eye(len(theta)) * oreml.RIDGE, base["grad"])
    assert float(base["grad"] @ d) > 0
    step = min(.002, .05 * float(np.min(theta / np.maximum(abs(d), 1e-9))))
    assert oreml.evaluate(ctx, theta + step * d)["ll"] > base["ll"]
