"""Matrix-free SLQ log-determinant values and exact parameter gradients.

Same contract as GPU_REML's slq.py:143-213.  Lanczos vectors live on the
device in FP32; the recurrence keeps two-pass full reorthogonalisation
against the basis (slq.py:49-74); the small tridiagonal eigenproblems, the
Gauss quadrature of log and its divided-difference derivative
(slq.py:84-121) run in FP64 on the device.  The gradient is the exact
derivative of the same fixed-probe value, obtained by a reverse pass over
the recurrence whose vector-Jacobian product is written out explicitly (the
reference obtains it with jax.vjp, slq.py:77-81); the reverse pass reuses the
caller's streamed ``matvec_pullback(left, right) -> (A left, grad)``.

Probe signs are drawn from a seeded torch generator (the reference uses
jax.random); the whole (n, nsamples) sign matrix is drawn once so that probe
batching does not change the target.
"""
from __future__ import annotations

import math

import torch

F32_EPS = float(torch.finfo(torch.float32).eps)


def default_workspace_bytes(gpu_budget_bytes=None):
    """slq.py:16-21"""
    return (
        min(2 * 1024 ** 3, max(1, int(gpu_budget_bytes / 8)))
        if gpu_budget_bytes is not None else 256 * 1024 ** 2
    )


def workspace_layout(n, nsamples, m, workspace_bytes, *, itemsize=4):
    """Probe batching policy (slq.py:24-41)."""
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


def rademacher(n: int, nsamples: int, seed: int, device, dtype=torch.float32) -> torch.Tensor:
    gen = torch.Generator(device="cpu")
    gen.manual_seed(int(seed))
    signs = torch.randint(0, 2, (n, nsamples), generator=gen, dtype=torch.int8)
    return (signs.to(dtype) * 2 - 1).to(device)


def _proj(P, w):
    return torch.einsum("ins,ns->is", P, w)


def _back(P, c):
    return torch.einsum("ins,is->ns", P, c)


def _forward(basis, product, prev_beta, index, eps):
    q = basis[index]
    prev = basis[index - 1] if index > 0 else torch.zeros_like(q)
    active = torch.sum(q * q, dim=0) > 0
    w0 = product - prev * prev_beta
    alpha = torch.sum(q * w0, dim=0)
    w1 = w0 - q * alpha
    P = basis[: index + 1]
    c1 = _proj(P, w1)
    w2 = w1 - _back(P, c1)
    c2 = _proj(P, w2)
    w3 = w2 - _back(P, c2)
    square = torch.sum(w3 * w3, dim=0)
    norm = torch.sqrt(torch.where(square > 0, square, torch.ones_like(square)))
    scale = torch.sqrt(torch.sum(product * product, dim=0))
    thr = 16 * eps * torch.maximum(scale, alpha.abs())
    keep = active & (square > thr * thr)
    beta = torch.where(keep, norm, torch.zeros_like(norm))
    nxt = torch.where(keep[None, :], w3 / torch.where(keep, norm, torch.ones_like(norm)),
                      torch.zeros_like(w3))
    alpha_out = torch.where(active, alpha, torch.ones_like(alpha))
    cache = dict(q=q, prev=prev, active=active, w0=w0, alpha=alpha, w1=w1, w2=w2, c1=c1, c2=c2,
                 norm=norm, keep=keep, nxt=nxt, P=P)
    return nxt, alpha_out, beta, cache


def _step(basis, product, previous_beta, index, eps=F32_EPS):
    """One two-pass orthogonalised Lanczos step (slq.py:49-74)."""
    nxt, a, b, _ = _forward(basis, product, previous_beta, index, eps)
    return nxt, a, b


def _step_pullback(basis, product, previous_beta, index, q_bar, a_bar, b_bar, eps=F32_EPS):
    """Vector-Jacobian product of ``_step`` w.r.t. (basis, product, previous_beta)."""
    _, _, _, c = _forward(basis, product, previous_beta, index, eps)
    P, nxt, norm, keep = c["P"], c["nxt"], c["norm"], c["keep"]
    dB = torch.zeros_like(basis)
    w3bar = torch.where(keep[None, :],
                        (q_bar - nxt * torch.sum(nxt * q_bar, dim=0)) / norm + b_bar * nxt,
                        torch.zeros_like(q_bar))
    d3 = _proj(P, w3bar)
    w2bar = w3bar - _back(P, d3)
    dB[: index + 1] -= c["c2"][:, None, :] * w3bar[None] + d3[:, None, :] * c["w2"][None]
    d2 = _proj(P, w2bar)
    w1bar = w2bar - _back(P, d2)
    dB[: index + 1] -= c["c1"][:, None, :] * w2bar[None] + d2[:, None, :] * c["w1"][None]
    q, alpha = c["q"], c["alpha"]
    abar = torch.where(c["active"], a_bar, torch.zeros_like(a_bar)) - torch.sum(q * w1bar, dim=0)
    w0bar = w1bar + abar * q
    dB[index] += -alpha * w1bar + abar * c["w0"]
    if index > 0:
        dB[index - 1] += -previous_beta * w0bar
    pb_bar = -torch.sum(c["prev"] * w0bar, dim=0)
    return dB, w0bar, pb_bar


def _quadrature(alphas, betas, weight, eps=F32_EPS):
    """Value and Frechet derivative of sum e1^T log(T) e1 (slq.py:84-121), FP64."""
    alphas = alphas.to(torch.float64)
    betas = betas.to(torch.float64)
    depth, S = alphas.shape
    dev = alphas.device
    T = torch.zeros((S, depth, depth), dtype=torch.float64, device=dev)
    idx = torch.arange(depth, device=dev)
    T[:, idx, idx] = alphas.T
    off = torch.arange(depth - 1, device=dev)
    if depth > 1:
        T[:, off + 1, off] = betas.T
        T[:, off, off + 1] = betas.T
    values, vectors = torch.linalg.eigh(T)
    floor = max(eps * depth, 1e-6)
    clipped = torch.clamp(values, min=floor)
    logv = torch.log(clipped)
    leading = vectors[:, 0, :]
    value = weight * torch.sum(leading * leading * logv)
    diff = values[:, :, None] - values[:, None, :]
    scale = torch.maximum(values.abs()[:, :, None], values.abs()[:, None, :])
    close = diff.abs() <= 8 * eps * torch.clamp(scale, min=floor)
    denom = torch.where(close, torch.ones_like(diff), diff)
    rel = (clipped[:, :, None] - clipped[:, None, :]) / clipped[:, None, :]
    nearby = rel.abs() < 0.5
    logdiff = torch.where(nearby, torch.log1p(torch.where(nearby, rel, torch.zeros_like(rel))),
                          logv[:, :, None] - logv[:, None, :])
    mid = 0.5 * (values[:, :, None] + values[:, None, :])
    deriv = torch.where(mid > floor, 1.0 / torch.clamp(mid, min=floor), torch.zeros_like(mid))
    divided = torch.where(close, deriv, logdiff / denom)
    spectral = divided * leading[:, :, None] * leading[:, None, :]
    grad = weight * (vectors @ spectral @ vectors.transpose(1, 2))
    a_bar = torch.diagonal(grad, dim1=1, dim2=2).T
    b_bar = 2 * grad[:, off, off + 1].T if depth > 1 else torch.zeros((0, S), dtype=torch.float64,
                                                                     device=dev)
    return value, a_bar, b_bar


def _batch_pullback(matvec_pullback, basis, products, beta, a_bar, b_bar, eps=F32_EPS):
    """Reverse an already computed Lanczos batch (slq.py:124-140)."""
    dt = basis.dtype
    q_bar = torch.zeros_like(basis)
    b_bar = b_bar.to(dt).clone()
    a_bar = a_bar.to(dt)
    zero = torch.zeros(basis.shape[2], dtype=dt, device=basis.device)
    gradient = None
    for index in range(products.shape[0] - 1, -1, -1):
        dB, dw, db = _step_pullback(basis, products[index], beta[index - 1] if index else zero,
                                    index, q_bar[index + 1], a_bar[index], b_bar[index], eps)
        q_bar = q_bar + dB
        input_bar, part = matvec_pullback(dw.contiguous(), basis[index].contiguous())
        q_bar[index] += input_bar
        part = torch.as_tensor(part, dtype=torch.float64, device=basis.device)
        gradient = part if gradient is None else gradient + part
        if index:
            b_bar[index - 1] += db
    return gradient


def logdet_value_and_grad(matvec, matvec_pullback, n, key, *, nsamples, m,
                          workspace_bytes=256 * 1024 ** 2, dtype=torch.float32,
                          accept_value=None, device=None, probes=None, eps=None):
    """Fixed-probe SLQ value and its exact parameter gradient (slq.py:143-213).

    ``key`` seeds the Rademacher probes unless ``probes`` (n, nsamples) are
    given.  Returns (value FP64 tensor, gradient FP64 tensor or None).
    """
    depth = min(int(m), int(n))
    itemsize = torch.empty((), dtype=dtype).element_size()
    eps = float(torch.finfo(dtype).eps) if eps is None else eps
    layout = workspace_layout(n, nsamples, m, workspace_bytes, itemsize=itemsize)
    width = layout["batch_width"]
    defer = (accept_value is not None and matvec_pullback is not None
             and layout["retained_bytes"] <= workspace_bytes)
    dev = device if device is not None else torch.device("cuda")
    if probes is None:
        probes = rademacher(n, nsamples, key, dev, dtype)
    probes = probes.to(device=dev, dtype=dtype)
    dev = probes.device
    pending = []
    total = torch.zeros((), dtype=torch.float64, device=dev)
    total_grad = None
    for start in range(0, nsamples, width):
        count = min(width, nsamples - start)
        basis = torch.zeros((depth + 1, n, count), dtype=dtype, device=dev)
        basis[0] = probes[:, start:start + count] / math.sqrt(n)
        products = None if matvec_pullback is None else torch.zeros((depth, n, count), dtype=dtype,
                                                                    device=dev)
        alphas, betas = [], []
        prev_beta = torch.zeros(count, dtype=dtype, device=dev)
        for index in range(depth):
            product = torch.as_tensor(matvec(basis[index].contiguous()), dtype=dtype, device=dev)
            nxt, a, b = _step(basis, product, prev_beta, index, eps)
            if products is not None:
                products[index] = product
            basis[index + 1] = nxt
            alphas.append(a)
            betas.append(b)
            prev_beta = b
        A = torch.stack(alphas)
        Bt = torch.stack(betas[:-1]) if depth > 1 else torch.zeros((0, count), dtype=dtype, device=dev)
        value, a_bar, b_small = _quadrature(A, Bt, n / nsamples, eps)
        total = total + value
        if matvec_pullback is None:
            del basis
            continue
        b_bar = torch.cat([b_small, torch.zeros((1, count), dtype=torch.float64, device=dev)])
        if defer:
            pending.append((basis, products, betas, a_bar, b_bar))
        else:
            g = _batch_pullback(matvec_pullback, basis, products, betas, a_bar, b_bar, eps)
            total_grad = g if total_grad is None else total_grad + g
        del basis, products
    if not bool(torch.isfinite(total)):
        raise FloatingPointError("Nonfinite SLQ value.")
    if accept_value is not None and not accept_value(total):
        return total, None
    for batch in pending:
        g = _batch_pullback(matvec_pullback, *batch, eps=eps)
        total_grad = g if total_grad is None else total_grad + g
    if total_grad is not None and not bool(torch.all(torch.isfinite(total_grad))):
        raise FloatingPointError("Nonfinite SLQ derivative.")
    return total, total_grad


__all__ = ["logdet_value_and_grad", "workspace_layout", "default_workspace_bytes", "rademacher"]
