"""Host FP64 pieces of the H^{-1} path (no GPU): projected H^{-1} vector,
SPD solve and the convergence gate."""
import numpy as np
import pytest

from coherit_gb300.hinv import compute_projected_hinv_vector, require_pcg_converged, solve_spd


def test_projected_hinv_vector_matches_formula():
    rng = np.random.default_rng(0)
    n, p = 50, 3
    A = rng.normal(size=(n, n))
    H = A @ A.T + n * np.eye(n)
    C = rng.normal(size=(n, p))
    t = rng.normal(size=n)
    Hi_t, Hi_C = np.linalg.solve(H, t), np.linalg.solve(H, C)
    got = compute_projected_hinv_vector(C, Hi_C, Hi_t, ridge=0.0)
    ref = Hi_t - Hi_C @ np.linalg.solve(C.T @ Hi_C, C.T @ Hi_t)
    np.testing.assert_allclose(got, ref, rtol=1e-10)
    # Projection property: C^T P_C t = 0.
    np.testing.assert_allclose(C.T @ got, 0.0, atol=1e-10)
    np.testing.assert_array_equal(compute_projected_hinv_vector(None, None, Hi_t), Hi_t)
    with pytest.raises(ValueError):
        compute_projected_hinv_vector(C, Hi_C[:, :2], Hi_t)


def test_solve_spd_and_gate():
    A = np.array([[4.0, 1.0], [1.0, 3.0]])
    b = np.array([1.0, 2.0])
    np.testing.assert_allclose(solve_spd(A, b), np.linalg.solve(A, b))
    assert solve_spd(np.zeros((0, 0)), np.zeros(0)).size == 0
    assert require_pcg_converged(1.0e-6, tol=1e-6, iters=3, maxiter=10, stage="s") == 1e-6
    with pytest.raises(RuntimeError, match="did not converge"):
        require_pcg_converged(1.1e-6, tol=1e-6, iters=3, maxiter=10, stage="s")
    with pytest.raises(RuntimeError):
        require_pcg_converged(float("nan"), tol=1e-6, iters=3, maxiter=10, stage="s")
