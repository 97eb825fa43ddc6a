"""Pin the CPU oracle to the known-answer checks of the reference's own tests.

Each test restates one check of the reference suite (file:line given) and
runs it against the oracle restatement.  The same checks run against the GPU
implementation in the gpu-marked tests.
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
