"""Lazy evaluation in the REML driver (tests/test_reml_lazy_evaluation.py of
the reference, lines 106-227), on CPU: dense kernels, and pcg_solve replaced
by an exact solve that counts its calls.  A trial rejected by the strict
line search costs one solve and no AI solve or SLQ reverse pass; an accepted
one reproduces the eager evaluation; lazy and eager fits follow the same
trajectory; failed trials raise or back off as the reference's do."""
import numpy as np
import pytest
import torch

from coherit_gb300 import reml, slq

CPU = torch.device("cpu")


def _exact_solve(Hv, B, M=None, tol=1e-2, maxiter=200, X0=None, check_every=2):
    B2 = torch.as_tensor(B).float()
    vec = B2.ndim == 1
    B2 = B2[:, None] if vec else B2
    H = torch.as_tensor(Hv(torch.eye(B2.shape[0]))).double()
    X = torch.linalg.solve(0.5 * (H + H.T), B2.double()).float()
    R = B2.double() - torch.as_tensor(Hv(X)).double()
    rel = torch.max(R.norm(dim=0) / B2.double().norm(dim=0).clamp_min(1e-300))
    return (X[:, 0] if vec else X), rel, 1


def _problem(groups=2):
    # tests/test_reml_lazy_evaluation.py:19-32 of the reference
    rng = np.random.default_rng(684)
    n = 24
    kernels = []
    for k in range(groups):
        x = rng.normal(size=(n, 12 + 5 * k)).astype(np.float32)
        kernels.append(torch.as_tensor(x @ x.T / x.shape[1] + .1 * np.eye(n), dtype=torch.float32))
    return dict(
        y=torch.as_tensor(rng.normal(size=n), dtype=torch.float32),
        K_mvs=tuple(lambda b, k=k: k @ b for k in kernels),
        diag_list=tuple(torch.diagonal(k) for k in kernels), covar=torch.ones((n, 1)),
        n_rand_vec=7, maxiter=100, minq_iter=1, slq_samples=4, slq_m=8,
        pcg_tol=1e-5, verbose=False, response_is_standardized=True, device="cpu",
    )


@pytest.fixture
def counted(monkeypatch):
    calls = {"solves": 0, "reverse": 0}

    def solve(*a, **kw):
        calls["solves"] += 1
        return _exact_solve(*a, **kw)

    original = slq._step_pullback

    def pullback(*a, **kw):
        calls["reverse"] += 1
        return original(*a, **kw)

    monkeypatch.setattr(reml, "pcg_solve", solve)
    monkeypatch.setattr(slq, "_step_pullback", pullback)
    return calls


@pytest.mark.parametrize("groups", [1, 2])
def test_rejected_trial_skips_ai_and_accepted_reproduces_eager(counted, groups):
    args = _problem(groups)
    theta = np.asarray([.2] * groups + [.6])
    y, c = args["y"], args["covar"]
    n = y.shape[0]
    rhs = torch.column_stack([c, y])
    ctx = reml.REMLContext(
        n=n, G=groups, E=1, K_mvs=args["K_mvs"], weighted_hv=None, stacked_kv=None,
        diag_stack=torch.stack(args["diag_list"]), residual_diag_stack=None, xmat=c, y=y,
        rhs_const=rhs, y_col=1, rand_stop=2, n_XyZ_cols=2, R_rand=0, kvrand_stack=None,
        precond_conf=None, residual_diag_atoms=np.ones(1))
    if groups == 1:
        ctx.affine_slq_cache = reml._build_affine_slq_cache(args["K_mvs"][0], n, 28, nsamples=4,
                                                            m=8, device=CPU)

    def evaluate(floor=None):
        return reml._eval_once(ctx, theta, torch.zeros_like(rhs), key_slq=28, minq_tol=1e-5,
                               maxiter=100, precond_eps=1e-6, slq_samples=4, slq_m=8,
                               compute_traces=False, min_loglik=floor)

    eager = evaluate()
    counted.update(solves=0, reverse=0)
    rejected = evaluate(eager[0] + 1)
    assert rejected[0] == eager[0]
    assert rejected[1] is None and rejected[2] is None
    assert counted == {"solves": 1, "reverse": 0}
    counted.update(solves=0, reverse=0)
    accepted = evaluate(eager[0])
    assert counted["solves"] == 2
    assert counted["reverse"] == (8 if groups > 1 else 0)
    assert accepted[0] == eager[0]
    for idx in (1, 4, 5):
        np.testing.assert_array_equal(np.asarray(accepted[idx]), np.asarray(eager[idx]))
    np.testing.assert_array_equal(np.asarray(accepted[8]), np.asarray(eager[8]))
    np.testing.assert_array_equal(accepted[2].mat, eager[2].mat)


def test_lazy_backtracking_matches_eager_trajectory(counted, monkeypatch):
    args = {**_problem(), "minq_iter": 3, "max_linesearch_trials": 8}
    original_direction = reml._projected_fisher_direction

    def overshoot(*a, **kw):
        direction, mask = original_direction(*a, **kw)
        return 8 * direction, mask

    monkeypatch.setattr(reml, "_projected_fisher_direction", overshoot)
    lazy = reml.fit_reml(**args)
    assert any(row["line_search_trials"] > 1 for row in lazy[1])
    original_eval = reml._eval_once

    def eager(*a, **kw):
        kw.pop("min_loglik", None)
        return original_eval(*a, **kw)

    monkeypatch.setattr(reml, "_eval_once", eager)
    full = reml.fit_reml(**args)
    np.testing.assert_array_equal(lazy[0], full[0])
    assert len(lazy[1]) == len(full[1])
    for first, second in zip(lazy[1], full[1]):
        for field in ("loglik", "params", "accepted", "line_search_trials", "stop_reason"):
            assert first.get(field) == second.get(field), field


def test_all_numerically_failed_trials_raise_instead_of_converging(counted, monkeypatch):
    original = reml._eval_once
    calls = 0

    def failing_trials(*args, **kwargs):
        nonlocal calls
        calls += 1
        if calls == 1:
            return original(*args, **kwargs)
        raise FloatingPointError("injected PCG failure")

    monkeypatch.setattr(reml, "_eval_once", failing_trials)
    with pytest.raises(FloatingPointError, match="could not evaluate any of 3 candidates") as err:
        reml.fit_reml(**_problem(), max_linesearch_trials=3)
    assert calls == 4
    assert "injected PCG failure" in str(err.value.__cause__)


@pytest.mark.parametrize("downhill", [False, True])
def test_numeric_failure_can_backtrack_to_a_finite_trial(counted, monkeypatch, downhill):
    original = reml._eval_once
    warmup = None
    calls = 0

    def mixed_trials(*args, **kwargs):
        nonlocal warmup, calls
        calls += 1
        if calls == 1:
            warmup = original(*args, **kwargs)
            return warmup
        if calls == 2:
            raise FloatingPointError("injected failed first trial")
        result = list(warmup)
        if downhill:
            result[0] = warmup[0] - 1.0
            result[1] = result[2] = None       # finite, lazily rejected objective
        return tuple(result)

    monkeypatch.setattr(reml, "_eval_once", mixed_trials)
    theta, history = reml.fit_reml(**_problem(), max_linesearch_trials=3)
    assert np.all(np.isfinite(theta))
    assert history[-1]["converged"]
    assert history[-1]["stop_reason"] == ("ll_down" if downhill else "rel_dll")
    assert history[-1]["accepted"] == (not downhill)
