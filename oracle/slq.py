"""Stochastic Lanczos quadrature restated in numpy (test infrastructure only).

* ``logdet_value_and_grad`` follows slq.py:143-213: fixed-probe SLQ with
  two-pass full reorthogonalisation (slq.py:49-74), the divided-difference
  quadrature and its Frechet derivative (slq.py:84-121), and the exact
  parameter gradient by a reverse pass over the recurrence (slq.py:77-81,
  :124-140).  The reference differentiates ``_step`` with jax.vjp; here its
  vector-Jacobian product is written out by hand (``step_vjp``).
* ``affine_cache`` / ``affine_logdet`` follow reml.py:285-304, :367-486: one
  Lanczos run on K with local orthogonalisation and the analytic logdet of
  theta_g T_K + theta_e I with its two derivatives.

Arithmetic is FP64; ``eps`` is the machine epsilon of the vector dtype the
reference would use (it sets the eigenvalue floor and breakdown tests).
"""
from __future__ import annotations

import numpy as np

F32_EPS = float(np.finfo(np.float32).eps)


def workspace_layout(n, nsamples, m, workspace_bytes, *, itemsize=4):
    """slq.py:24-41"""
    if n < 1 or nsamples < 1 or m < 1 or workspace_bytes < 1:
        raise ValueError("SLQ dimensions and workspace budget must be positive.")
    depth = min(int(m), int(n))
    per_probe = itemsize * n * (8 * (depth + 1) + 32)
    capacity = max(1, int(workspace_bytes) // per_probe)
    width = min(int(nsamples), 1 << (capacity.bit_length() - 1))
    retained = itemsize * n * (nsamples * (2 * depth + 1) + width * (6 * (depth + 1) + 32))
    eager = per_probe * width
    peak = max(eager, retained) if retained <= workspace_bytes else eager
    peak += 8 * itemsize * width * depth * depth
    return dict(batch_width=width, retained_bytes=retained, peak_bytes=peak)


def _forward(basis, product, prev_beta, index, eps):
    q = basis[index]
    prev = basis[index - 1] if index > 0 else np.zeros_like(q)
    active = np.sum(q * q, axis=0) > 0
    w0 = product - prev * prev_beta
    alpha = np.sum(q * w0, axis=0)
    w1 = w0 - q * alpha
    P = basis[: index + 1]
    c1 = np.einsum("ins,ns->is", P, w1)
    w2 = w1 - np.einsum("ins,is->ns", P, c1)
    c2 = np.einsum("ins,ns->is", P, w2)
    w3 = w2 - np.einsum("ins,is->ns", P, c2)
    square = np.sum(w3 * w3, axis=0)
    norm = np.sqrt(np.where(square > 0, square, 1.0))
    scale = np.sqrt(np.sum(product * product, axis=0))
    thr = 16 * eps * np.maximum(scale, np.abs(alpha))
    keep = active & (square > thr * thr)
    beta = np.where(keep, norm, 0.0)
    nxt = np.where(keep[None, :], w3 / np.where(keep, norm, 1.0), 0.0)
    cache = dict(q=q, prev=prev, active=active, w0=w0, alpha=alpha, w1=w1, w2=w2, w3=w3,
                 c1=c1, c2=c2, norm=norm, keep=keep, nxt=nxt, P=P)
    return nxt, np.where(active, alpha, 1.0), beta, cache


def step(basis, product, prev_beta, index, eps=F32_EPS):
    nxt, a, b, _ = _forward(basis, product, prev_beta, index, eps)
    return nxt, a, b


def step_vjp(basis, product, prev_beta, index, q_bar, a_bar, b_bar, eps=F32_EPS):
    """Cotangents of (basis, product, prev_beta) for one Lanczos step."""
    _, _, _, c = _forward(basis, product, prev_beta, index, eps)
    P, nxt, norm, keep = c["P"], c["nxt"], c["norm"], c["keep"]
    dB = np.zeros_like(basis)
    w3bar = np.where(
        keep[None, :], (q_bar - nxt * np.sum(nxt * q_bar, axis=0)) / norm + b_bar * nxt, 0.0)
    d3 = np.einsum("ins,ns->is", P, w3bar)
    w2bar = w3bar - np.einsum("ins,is->ns", P, d3)
    dB[: index + 1] -= c["c2"][:, None, :] * w3bar[None] + d3[:, None, :] * c["w2"][None]
    d2 = np.einsum("ins,ns->is", P, w2bar)
    w1bar = w2bar - np.einsum("ins,is->ns", P, d2)
    dB[: index + 1] -= c["c1"][:, None, :] * w2bar[None] + d2[:, None, :] * c["w1"][None]
    q, alpha = c["q"], c["alpha"]
    w0bar = w1bar.copy()
    qbar = -alpha * w1bar
    abar = np.where(c["active"], a_bar, 0.0) - np.sum(q * w1bar, axis=0)
    w0bar = w0bar + abar * q
    qbar = qbar + abar * c["w0"]
    dB[index] += qbar
    if index > 0:
        dB[index - 1] += -prev_beta * w0bar
    pb_bar = -np.sum(c["prev"] * w0bar, axis=0)
    return dB, w0bar, pb_bar


def quadrature(alphas, betas, weight, eps=F32_EPS):
    """Value and derivatives w.r.t. the tridiagonal entries (slq.py:84-121)."""
    depth, S = alphas.shape
    T = np.zeros((S, depth, depth))
    idx = np.arange(depth)
    T[:, idx, idx] = alphas.T
    off = np.arange(depth - 1)
    if depth > 1:
        T[:, off + 1, off] = betas.T
        T[:, off, off + 1] = betas.T
    values, vectors = np.linalg.eigh(T)
    floor = max(eps * depth, 1e-6)
    clipped = np.maximum(values, floor)
    logv = np.log(clipped)
    leading = vectors[:, 0, :]
    value = weight * np.sum(leading * leading * logv)
    diff = values[:, :, None] - values[:, None, :]
    scale = np.maximum(np.abs(values[:, :, None]), np.abs(values[:, None, :]))
    close = np.abs(diff) <= 8 * eps * np.maximum(scale, floor)
    denom = np.where(close, 1.0, diff)
    rel = (clipped[:, :, None] - clipped[:, None, :]) / clipped[:, None, :]
    nearby = np.abs(rel) < 0.5
    logdiff = np.where(nearby, np.log1p(np.where(nearby, rel, 0.0)),
                       logv[:, :, None] - logv[:, None, :])
    mid = 0.5 * (values[:, :, None] + values[:, None, :])
    deriv = np.where(mid > floor, 1.0 / np.maximum(mid, floor), 0.0)
    divided = np.where(close, deriv, logdiff / denom)
    spectral = divided * leading[:, :, None] * leading[:, None, :]
    grad = weight * (vectors @ spectral @ np.swapaxes(vectors, 1, 2))
    a_bar = np.diagonal(grad, axis1=1, axis2=2).T
    b_bar = 2 * grad[:, off, off + 1].T if depth > 1 else np.zeros((0, S))
    return value, a_bar, b_bar


def batch_pullback(matvec_pullback, basis, products, beta, a_bar, b_bar, eps=F32_EPS):
    """slq.py:124-140"""
    q_bar = np.zeros_like(basis)
    b_bar = np.array(b_bar, copy=True)
    gradient = None
    zero = np.zeros(basis.shape[2])
    for index in range(products.shape[0] - 1, -1, -1):
        dB, dw, db = step_vjp(basis, products[index], beta[index - 1] if index else zero, index,
                              q_bar[index + 1], a_bar[index], b_bar[index], eps)
        q_bar = q_bar + dB
        input_bar, part = matvec_pullback(dw, basis[index])
        q_bar[index] += input_bar
        gradient = part if gradient is None else gradient + part
        if index:
            b_bar[index - 1] += db
    return gradient


def logdet_value_and_grad(matvec, matvec_pullback, n, probes, *, m,
                          workspace_bytes=256 * 1024 ** 2, itemsize=4, accept_value=None,
                          eps=F32_EPS):
    """Fixed-probe SLQ value and gradient (slq.py:143-213); probes: (n, S) signs."""
    probes = np.asarray(probes, np.float64)
    nsamples = probes.shape[1]
    depth = min(int(m), int(n))
    layout = workspace_layout(n, nsamples, m, workspace_bytes, itemsize=itemsize)
    width = layout["batch_width"]
    defer = (accept_value is not None and matvec_pullback is not None
             and layout["retained_bytes"] <= workspace_bytes)
    pending = []
    total, total_grad = 0.0, None
    for start in range(0, nsamples, width):
        count = min(width, nsamples - start)
        basis = np.zeros((depth + 1, n, count))
        basis[0] = probes[:, start:start + count] / np.sqrt(n)
        products = None if matvec_pullback is None else np.zeros((depth, n, count))
        alphas, betas = [], []
        prev_beta = np.zeros(count)
        for index in range(depth):
            product = np.asarray(matvec(basis[index]), np.float64)
            nxt, a, b = step(basis, product, prev_beta, index, eps)
            if products is not None:
                products[index] = product
            basis[index + 1] = nxt
            alphas.append(a)
            betas.append(b)
            prev_beta = b
        A = np.stack(alphas)
        Bt = np.stack(betas[:-1]) if depth > 1 else np.zeros((0, count))
        value, a_bar, b_small = quadrature(A, Bt, n / nsamples, eps)
        total += value
        if matvec_pullback is None:
            continue
        b_bar = np.concatenate([b_small, np.zeros((1, count))])
        if defer:
            pending.append((basis, products, betas, a_bar, b_bar))
        else:
            g = batch_pullback(matvec_pullback, basis, products, betas, a_bar, b_bar, eps)
            total_grad = g if total_grad is None else total_grad + g
    if not np.isfinite(total):
        raise FloatingPointError("Nonfinite SLQ value.")
    if accept_value is not None and not accept_value(total):
        return total, None
    for batch in pending:
        g = batch_pullback(matvec_pullback, *batch, eps=eps)
        total_grad = g if total_grad is None else total_grad + g
    if total_grad is not None and not np.all(np.isfinite(total_grad)):
        raise FloatingPointError("Nonfinite SLQ derivative.")
    return total, total_grad


# --------------------------------------------------------------- affine SLQ

def affine_cache(K_fn, n, probes, m):
    """Lanczos on K with local orthogonalisation only (reml.py:285-304, :367-412)."""
    z = np.asarray(probes, np.float64)
    S = z.shape[1]
    v = z / np.sqrt(float(n))
    prev = np.zeros_like(v)
    beta_prev = np.zeros(S)
    alphas, betas = [], []
    for i in range(m):
        w = np.asarray(K_fn(v), np.float64) - prev * beta_prev
        alpha = np.sum(v * w, axis=0)
        w = w - v * alpha
        norm = np.linalg.norm(w, axis=0)
        v_next = w / np.where(norm > 0, norm, 1.0)
        alphas.append(alpha)
        if i < m - 1:
            betas.append(norm)
        prev, beta_prev, v = v, norm, v_next
    return dict(alphas=np.stack(alphas), betas=np.stack(betas) if betas else np.zeros((0, S)),
                z_norm_sq=float(n), nsamples=float(S))


def affine_logdet(cache, theta_g, theta_e, eps=F32_EPS):
    """logdet(theta_g K + theta_e I) and (d/dtheta_g, d/dtheta_e) (reml.py:415-486)."""
    A, B = cache["alphas"], cache["betas"]
    m, S = A.shape
    T = np.zeros((S, m, m))
    idx = np.arange(m)
    T[:, idx, idx] = A.T
    if m > 1:
        off = np.arange(m - 1)
        T[:, off + 1, off] = B.T
        T[:, off, off + 1] = B.T
    ev, vec = np.linalg.eigh(T)
    w = vec[:, 0, :] ** 2
    raw = theta_g * ev + theta_e
    floor = max(eps * m, 1e-6)
    h = np.maximum(raw, floor)
    active = (raw > floor).astype(float)
    factor = cache["z_norm_sq"] / cache["nsamples"]
    logdet = factor * np.sum(w * np.log(h))
    d_scale = factor * np.sum(w * active * ev / h)
    d_shift = factor * np.sum(w * active / h)
    return logdet, np.asarray([d_scale, d_shift])
