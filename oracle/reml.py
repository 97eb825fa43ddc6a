"""REML evaluation and strict AI-REML fit restated in numpy (test infrastructure only).

Follows reml.py of the reference: response standardisation (:151-163),
_eval_once (:685-971) with the affine single-GRM SLQ (:367-486) or the
multi-component SLQ with its exact score (:489-540), the fixed-effect
projection through the Cholesky of X^T H^-1 X (:780-801), the bounded Fisher
step by NNLS + KKT polish (:979-1247), the strict line search of fit_reml
(:1695-1880) and its one-trial scoring optimizer with Hutchinson traces
(:608-649, :1798-1808, :1909-1911).  Operators are numpy callables; vectors
are FP64.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
from scipy.optimize import nnls

from . import pcg as opcg
from . import precond as oprec
from . import slq as oslq

RIDGE = 1e-4


def standardize(y):
    y = np.asarray(y, np.float32).reshape(-1)
    mu = np.mean(y, dtype=np.float32)
    sd = np.std(y, dtype=np.float32)
    return ((y - mu) / (sd + np.float32(1e-6))).astype(np.float32), float(mu), float(sd + 1e-6)


def stable_chol(A, base=1e-6, tries=8):
    A = 0.5 * (A + A.T)
    scale = float(np.mean(np.abs(np.diag(A)))) or 1.0
    for k in range(-1, tries):
        jit = 0.0 if k < 0 else base * scale * 10.0 ** k
        try:
            L = np.linalg.cholesky(A + jit * np.eye(A.shape[0]))
            if np.all(np.isfinite(np.diag(L))) and np.all(np.diag(L) > 0):
                return L
        except np.linalg.LinAlgError:
            pass
    raise FloatingPointError("Failed to stabilize XtHinvX Cholesky with jitter escalation.")


class Context:
    """Inputs of one REML objective (reml.py:76-100), numpy flavour."""

    def __init__(self, y, K_list, X=None, *, diag_atoms=None, slq_probes=None, slq_m=30,
                 affine_cache=None, precond=None, pcg_tol=1e-6, maxiter=500, precond_eps=1e-6,
                 residual_diags=None, trace_probes=None):
        self.y = np.asarray(y, np.float64)
        self.n = self.y.size
        self.K = list(K_list)                  # callables on (n, k) arrays
        self.G = len(self.K)
        self.R = None if residual_diags is None else np.asarray(residual_diags, np.float64)
        self.E = 1 if self.R is None else self.R.shape[0]
        self.X = None if X is None else np.asarray(X, np.float64)
        self.diag_atoms = np.ones(self.G) if diag_atoms is None else np.asarray(diag_atoms, float)
        self.slq_probes = slq_probes
        self.slq_m = slq_m
        self.affine = affine_cache
        self.precond = precond
        self.pcg_tol = pcg_tol
        self.maxiter = maxiter
        self.precond_eps = precond_eps
        self.trace_probes = trace_probes
        parts = [] if self.X is None else [self.X]
        parts.append(self.y[:, None])
        if trace_probes is not None:
            parts.append(np.asarray(trace_probes, np.float64))
        self.rhs = np.concatenate(parts, axis=1)
        self.y_col = 0 if self.X is None else self.X.shape[1]

    def hv(self, theta):
        G = self.G

        def f(V):
            V = np.asarray(V, np.float64)
            if self.R is None:
                acc = theta[G] * V
            else:
                d = np.tensordot(theta[G:], self.R, axes=1)
                acc = d[:, None] * V if V.ndim == 2 else d * V
            for i, K in enumerate(self.K):
                if theta[i] != 0:
                    acc = acc + theta[i] * K(V)
            return acc
        return f

    def residual_products(self, V):
        if self.R is None:
            return [V]
        return [self.R[e][:, None] * V for e in range(self.E)]


def evaluate(ctx: Context, theta, *, warm=None, min_loglik=None, taylor=None):
    """One REML objective, score and AI matrix (reml.py:685-971)."""
    theta = np.asarray(theta, np.float64)
    G, n = ctx.G, ctx.n
    Hv = ctx.hv(theta)
    diag = float(np.dot(theta[G:], np.ones(ctx.E) if ctx.R is None else ctx.R.mean(axis=1))
                 + np.dot(theta[:G], ctx.diag_atoms))
    M = None
    if ctx.precond is not None:
        rt = oprec.runtime(ctx.precond, theta[:G], diag, ctx.precond_eps)
        M = lambda v: oprec.apply_inverse(rt, v)
    X0 = warm if warm is not None else (M(ctx.rhs) if M is not None else None)
    sol, rel, k = opcg.pcg_solve(lambda v: Hv(v).astype(np.float32), ctx.rhs.astype(np.float32),
                                 M=(None if M is None else (lambda v: M(v).astype(np.float32))),
                                 tol=ctx.pcg_tol, maxiter=ctx.maxiter, X0=X0)
    if not math.isfinite(rel) or rel > ctx.pcg_tol * 1.05:
        raise FloatingPointError(f"Main REML PCG did not converge: relative residual={rel:.3e}")
    sol = sol.astype(np.float64)
    chol = None
    if ctx.X is not None:
        p = ctx.X.shape[1]
        HinvX = sol[:, :p]
        chol = stable_chol(ctx.X.T @ HinvX)
        proj = lambda mat: mat - HinvX @ sla.cho_solve((chol, True), ctx.X.T @ mat)
    else:
        HinvX = None
        proj = lambda mat: mat
    PY = proj(sol[:, ctx.y_col:])
    Py = PY[:, :1]
    yPy = float(ctx.y @ PY[:, 0])
    logdet_x = 2.0 * np.sum(np.log(np.clip(np.diag(chol), 1e-30, None))) if chol is not None else 0.0
    ll_of = lambda ld: -0.5 * (yPy + ld + logdet_x) / n
    if taylor is not None:
        logdet, tr = taylor, None
    elif ctx.affine is not None:
        logdet, tr = oslq.affine_logdet(ctx.affine, theta[0], theta[1])
    else:
        def pullback(left, right):
            res = np.zeros_like(left)
            scores = []
            for i, K in enumerate(ctx.K):
                prod = K(left)
                res = res + theta[i] * prod
                scores.append(np.sum(right * prod))
            for e, prod in enumerate(ctx.residual_products(left)):
                res = res + theta[G + e] * prod
                scores.append(np.sum(right * prod))
            return res, np.asarray(scores)
        accept = None if min_loglik is None else (lambda v: ll_of(v) >= min_loglik)
        logdet, tr = oslq.logdet_value_and_grad(Hv, pullback, n, ctx.slq_probes, m=ctx.slq_m,
                                                accept_value=accept)
    ll = ll_of(logdet)
    if not math.isfinite(ll):
        raise FloatingPointError("Non-finite REML objective.")
    if min_loglik is not None and not ll >= min_loglik:
        return dict(ll=ll, grad=None, ai=None, sol=sol, logdet=logdet, pcg=k)
    GPy = [K(Py)[:, 0] for K in ctx.K] + [r[:, 0] for r in ctx.residual_products(Py)]
    GPy = np.stack(GPy, axis=1)
    q = Py[:, 0] @ GPy
    if taylor is not None:
        Vr = np.asarray(ctx.trace_probes, np.float64)
        PZ = PY[:, 1:]
        trg = np.asarray([np.sum(PZ * K(Vr)) for K in ctx.K]) / Vr.shape[1]
        trr = np.asarray([np.sum(Vr * P) for P in ctx.residual_products(PZ)]) / Vr.shape[1]
        tr = np.concatenate([trg, trr])
    elif HinvX is not None:
        rhs = [HinvX.T @ K(HinvX) for K in ctx.K] + [HinvX.T @ P for P in ctx.residual_products(HinvX)]
        corr = np.asarray([np.trace(sla.cho_solve((chol, True), r)) for r in rhs])
        tr = tr - corr
    X0a = M(GPy) if M is not None else None
    HG, rel_a, _ = opcg.pcg_solve(lambda v: Hv(v).astype(np.float32), GPy.astype(np.float32),
                                  M=(None if M is None else (lambda v: M(v).astype(np.float32))),
                                  tol=ctx.pcg_tol, maxiter=ctx.maxiter, X0=X0a)
    if not math.isfinite(rel_a) or rel_a > ctx.pcg_tol * 1.05:
        raise FloatingPointError("Average-information PCG did not converge")
    PG = proj(HG.astype(np.float64))
    AI = 0.5 * GPy.T @ PG / n
    AI = 0.5 * (AI + AI.T)
    grad = 0.5 * (q - tr) / n
    return dict(ll=ll, grad=grad, ai=AI, sol=sol, logdet=logdet, pcg=k)


def fisher_step(param, grad, ai, *, G, zero_tol=1e-8, floor=1e-2, alpha=1.0, ridge=RIDGE):
    """Bounded Fisher direction by NNLS + KKT polish (reml.py:979-1221)."""
    param = np.asarray(param, float)
    grad = np.asarray(grad, float)
    n_p = param.size
    lower = (np.concatenate([np.zeros(G), np.full(n_p - G, floor)]) - param) / alpha
    system = 0.5 * (ai + ai.T) + ridge * np.eye(n_p)
    scale = float(np.mean(np.abs(np.diag(system)))) or 1.0
    for a in range(9):
        jit = 0.0 if a == 0 else 1e-8 * scale * 10.0 ** (a - 1)
        try:
            L = np.linalg.cholesky(system + jit * np.eye(n_p))
            system = system + jit * np.eye(n_p)
            break
        except np.linalg.LinAlgError:
            continue
    rhs = grad - system @ lower
    x, _ = nnls(L.T, sla.solve_triangular(L, rhs, lower=True), maxiter=max(3 * n_p, 1))
    act = alpha * x <= max(zero_tol, 1e-10)
    kkt_tol = max(1e-7, 1e-6 * max(1.0, float(np.max(np.abs(grad)))))
    for _ in range(max(5 * n_p, 1)):
        x[:] = 0.0
        free = ~act
        if np.any(free):
            x[free] = np.linalg.solve(system[np.ix_(free, free)], rhs[free])
            bad = free & (x <= 0)
            if np.any(bad):
                act[bad] = True
                continue
        r = rhs - system @ x
        viol = act & (r > kkt_tol)
        if np.any(viol):
            c = np.flatnonzero(viol)
            act[c[np.argmax(r[c])]] = False
            continue
        break
    return lower + x


def apply_step(param, d, alpha, *, G, zero_tol=1e-8, floor=1e-2):
    tg = np.maximum(param[:G] + alpha * d[:G], 0.0)
    tg = np.where(tg <= zero_tol, 0.0, tg)
    return np.concatenate([tg, np.maximum(param[G:] + alpha * d[G:], floor)])


def fit(ctx: Context, *, h2_init=0.5, minq_iter=50, trials=3, rel_dll_tol=1e-3, floor=1e-2):
    """Strict AI-REML with backtracking (reml.py:1465-1880)."""
    G, E = ctx.G, ctx.E
    ra = np.ones(E) if ctx.R is None else ctx.R.mean(axis=1)
    param = np.concatenate([np.where(ctx.diag_atoms > 0, h2_init / np.sum(ctx.diag_atoms), 0.0),
                            np.maximum(np.full(E, (1 - h2_init) / np.sum(ra)), floor)])
    cur = evaluate(ctx, param)
    history = []
    for it in range(minq_iter):
        alpha = 1.0
        accepted = None
        for _ in range(trials):
            d = fisher_step(param, cur["grad"], cur["ai"], G=G, floor=floor, alpha=alpha)
            cand = apply_step(param, d, alpha, G=G, floor=floor)
            try:
                res = evaluate(ctx, cand, warm=cur["sol"], min_loglik=cur["ll"])
            except FloatingPointError:
                alpha *= 0.5
                continue
            if res["ll"] - cur["ll"] >= 0:
                accepted = (cand, res)
                break
            alpha *= 0.5
        if accepted is None:
            history.append(dict(iter=it + 1, accepted=False, params=list(param)))
            break
        cand, res = accepted
        rel = (res["ll"] - cur["ll"]) / max(abs(cur["ll"]), 1e-12)
        param, cur = cand, res
        history.append(dict(iter=it + 1, accepted=True, loglik=cur["ll"], params=list(param)))
        if rel < rel_dll_tol:
            break
    return param, history, cur


def hutchinson_traces(ctx: Context, sol):
    """tr(H^-1 K_i) and tr(H^-1 R_j) estimated from the trace-probe columns of
    a solve, (1/R) sum_r (H^-1 z_r)^T (K_i z_r) (reml.py:608-649)."""
    Z = np.asarray(ctx.trace_probes, np.float64)
    R = Z.shape[1]
    a = ctx.y_col + 1
    HZ = np.asarray(sol, np.float64)[:, a:a + R]
    trK = np.asarray([np.sum(HZ * K(Z)) for K in ctx.K]) / R
    trR = np.asarray([np.sum(Z * P) for P in ctx.residual_products(HZ)]) / R
    return trK, trR


def fit_scoring(ctx: Context, *, h2_init=0.5, minq_iter=50, taylor_threshold=0.01,
                scoring_step_tol=1e-4, floor=1e-2):
    """The ``smile_scoring`` optimizer of fit_reml (reml.py:1760-1911): one
    trial per iteration at alpha = 1, every step accepted; when the largest
    relative parameter change is below ``taylor_threshold`` the trial's
    log-determinant is the first-order expansion logdet + dtheta . traces
    (traces from the trace-probe columns of the last accepted solve) and its
    score comes from the Hutchinson traces of the projected probes; stop when
    that change is below ``scoring_step_tol``.  Needs ``ctx.trace_probes``."""
    if ctx.trace_probes is None:
        raise ValueError("the scoring optimizer needs trace probes")
    G, E = ctx.G, ctx.E
    ra = np.ones(E) if ctx.R is None else ctx.R.mean(axis=1)
    param = np.concatenate([np.where(ctx.diag_atoms > 0, h2_init / np.sum(ctx.diag_atoms), 0.0),
                            np.maximum(np.full(E, (1 - h2_init) / np.sum(ra)), floor)])
    cur = evaluate(ctx, param)
    trK, trR = hutchinson_traces(ctx, cur["sol"])
    logdet_c = cur["logdet"]
    history = []
    for it in range(minq_iter):
        d = fisher_step(param, cur["grad"], cur["ai"], G=G, floor=floor, alpha=1.0)
        cand = apply_step(param, d, 1.0, G=G, floor=floor)
        delta = cand - param
        max_rel_dp = float(np.max(np.abs(delta) / np.maximum(np.abs(param), 1e-8)))
        taylor = None
        if max_rel_dp < taylor_threshold:
            taylor = float(logdet_c + delta[:G] @ trK + delta[G:] @ trR)
        res = evaluate(ctx, cand, warm=cur["sol"], taylor=taylor)
        rel = (res["ll"] - cur["ll"]) / max(abs(cur["ll"]), 1e-12)
        trK, trR = hutchinson_traces(ctx, res["sol"])
        logdet_c = res["logdet"]
        param, cur = cand, res
        history.append(dict(iter=it + 1, loglik=cur["ll"], params=list(param),
                            taylor=taylor is not None, max_rel_dp=max_rel_dp))
        if not math.isfinite(rel) or max_rel_dp < scoring_step_tol:
            break
    return param, history, cur


def heritability(param, G, genetic_atoms, residual_atoms=(1.0,)):
    """h2 = sum theta_g a / (sum theta_g a + sum theta_e b) (reml_model.py:1945-1953)."""
    gen = float(np.dot(param[:G], genetic_atoms))
    res = float(np.dot(param[G:], residual_atoms))
    return gen / max(gen + res, 1e-8)
