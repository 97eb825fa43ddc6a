"""Projected-core preconditioner ``M = d I + U C U^T`` (precond.py of GPU_REML).

For an orthonormal basis U (n x r) the inverse and inverse square root act
on the r-dimensional projection only:
    M^{-1} v    = d^{-1} v + U ((dI + C)^{-1} - d^{-1} I) U^T v      (precond.py:42-58)
    M^{-1/2} v  = d^{-1/2} v + U ((dI + C)^{-1/2} - d^{-1/2} I) U^T v (precond.py:61-84)
On the GPU both applies run as one library call, out = a V + U (G (U^T V))
(coherit_lowrank_apply: the two n-long contractions and the r x r product
in the library's own kernels), with the r x r core G formed once per
factorisation; host tensors take the explicit formulas above.  The r x r
factorisations (Cholesky, eigh) are cuSOLVER calls.  The Nystrom basis
takes two operator applications on n x (r + 8) blocks (precond.py:251-276).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional

import torch


@dataclass
class ProjectedCorePrecondConf:
    """Shared basis + per-component projected cores (precond.py:15-26)."""

    U: torch.Tensor                       # (n, r) orthonormal basis
    core_atoms: torch.Tensor              # (G, r, r)
    total_rank: int
    n_grm: int
    diag_mode: Optional[str] = None       # "scalar_identity"
    diag_atoms: Optional[torch.Tensor] = None
    residual_diag_atoms: Optional[torch.Tensor] = None
    identity: Optional[torch.Tensor] = None


@dataclass
class ProjectedCoreRuntime:
    """Theta-specific factorisation (precond.py:29-39).  On the GPU also the
    r x r cores of the fused apply: G = (dI + C)^{-1} - d^{-1} I and, with
    the eigendecomposition, Q diag(e^{-1/2}) Q^T - d^{-1/2} I, with their
    scalars 1/d and d^{-1/2} as host floats."""

    U: torch.Tensor
    total_rank: int
    d: torch.Tensor
    d_inv: torch.Tensor
    chol: torch.Tensor
    eigvals: Optional[torch.Tensor] = None
    eigvecs: Optional[torch.Tensor] = None
    core_inv: Optional[torch.Tensor] = None
    core_invsqrt: Optional[torch.Tensor] = None
    a_inv: float = 0.0
    a_invsqrt: float = 0.0


def _lowrank_apply(v, U, G, a: float):
    """a v + U (G (U^T v)) in one library call (coherit_lowrank_apply)."""
    import ctypes as C

    from . import _lib

    vec = v.ndim == 1
    V = (v[:, None] if vec else v).to(torch.float32).contiguous()
    n, k = V.shape
    r = U.shape[1]
    lib = _lib.load()
    floats = C.c_int64()
    _lib.check(lib.coherit_lowrank_workspace_floats(n, r, k, C.byref(floats)), "low-rank apply")
    work = torch.empty(int(floats.value), dtype=torch.float32, device=V.device)
    out = torch.empty_like(V)
    _lib.check(lib.coherit_lowrank_apply(n, r, k, U.data_ptr(), U.stride(0), G.data_ptr(),
                                         G.stride(0), float(a), V.data_ptr(), V.stride(0),
                                         out.data_ptr(), out.stride(0), work.data_ptr(),
                                         int(floats.value), _lib.stream_ptr()), "low-rank apply")
    return out[:, 0] if vec else out


def _apply_scalar_diag(v: torch.Tensor, d_inv, chol, U) -> torch.Tensor:
    vec = v.ndim == 1
    V = v[:, None] if vec else v
    rhs = U.T @ V
    z = torch.cholesky_solve(rhs, chol, upper=False)
    out = d_inv * V + U @ (z - d_inv * rhs)
    return out[:, 0] if vec else out


def _apply_invsqrt(v, d_inv_sqrt, eigvals, eigvecs, U):
    vec = v.ndim == 1
    V = v[:, None] if vec else v
    rhs = U.T @ V
    coeff = eigvecs.T @ rhs
    scaled = coeff / torch.sqrt(torch.clamp(eigvals, min=1e-8))[:, None]
    z = eigvecs @ scaled
    out = d_inv_sqrt * V + U @ (z - d_inv_sqrt * rhs)
    return out[:, 0] if vec else out


def _scalar_diag_value(diag_H, dtype, device) -> torch.Tensor:
    arr = torch.as_tensor(diag_H, dtype=dtype, device=device)
    if arr.ndim == 0:
        return arr
    if arr.numel() != 1:
        raise ValueError("Projected-core MVP currently requires a scalar diagonal base.")
    return arr.reshape(())


def scalar_diag_from_precond_conf(precond_conf, theta_g, theta_e):
    """d = theta_e . residual_atoms + theta_g . diag_atoms (precond.py:96-118)."""
    if precond_conf is None or precond_conf.diag_mode != "scalar_identity":
        return None
    theta_g = torch.as_tensor(theta_g)
    dev = theta_g.device
    if precond_conf.diag_atoms is None:
        diag_atoms = torch.ones(precond_conf.n_grm, dtype=theta_g.dtype, device=dev)
    else:
        diag_atoms = torch.as_tensor(precond_conf.diag_atoms, dtype=theta_g.dtype, device=dev)
    te = torch.as_tensor(theta_e, dtype=theta_g.dtype, device=dev).reshape(-1)
    if precond_conf.residual_diag_atoms is None:
        ra = torch.ones(te.shape[0], dtype=theta_g.dtype, device=dev)
    else:
        ra = torch.as_tensor(precond_conf.residual_diag_atoms, dtype=theta_g.dtype,
                             device=dev).reshape(-1)
        if ra.shape[0] != te.shape[0]:
            raise ValueError(
                "Projected-core residual_diag_atoms length mismatch: "
                f"expected {te.shape[0]}, got {ra.shape[0]}."
            )
    return torch.dot(te, ra) + torch.dot(theta_g.reshape(-1), diag_atoms)


def build_projected_core_runtime(precond_conf, theta_g, diag_H, eps: float = 0.0, *,
                                 need_invsqrt: bool = False) -> Optional[ProjectedCoreRuntime]:
    """Assemble and factorise dI + sum_g theta_g C_g (precond.py:121-171)."""
    if precond_conf is None:
        return None
    if precond_conf.U.numel() == 0 or precond_conf.total_rank <= 0:
        return None
    if precond_conf.diag_mode != "scalar_identity":
        raise NotImplementedError(
            "Projected-core preconditioner currently supports only diag_mode='scalar_identity'."
        )
    U = precond_conf.U
    tg = torch.as_tensor(theta_g, dtype=U.dtype, device=U.device).reshape(-1)
    core = torch.tensordot(tg, precond_conf.core_atoms.to(U.dtype), dims=1)
    core = 0.5 * (core + core.T)
    d = _scalar_diag_value(diag_H, U.dtype, U.device) + eps
    d = torch.clamp(d, min=1e-8)
    r = precond_conf.total_rank
    if precond_conf.identity is None:
        identity = torch.eye(r, dtype=U.dtype, device=U.device)
    else:
        identity = precond_conf.identity.to(U.dtype)
        if tuple(identity.shape) != (r, r):
            raise ValueError(
                f"Projected-core identity cache shape mismatch: expected {(r, r)}, "
                f"got {tuple(identity.shape)}."
            )
    middle = core + d * identity
    chol = torch.linalg.cholesky(middle)
    eigvals = eigvecs = None
    if need_invsqrt:
        ev, eigvecs = torch.linalg.eigh(middle)
        eigvals = torch.clamp(ev, min=1e-8)
    rt = ProjectedCoreRuntime(U=U, total_rank=r, d=d, d_inv=1.0 / d, chol=chol,
                              eigvals=eigvals, eigvecs=eigvecs)
    if U.is_cuda and U.dtype == torch.float32 and U.is_contiguous():
        fused_cores(rt)
    return rt


def fused_cores(rt: ProjectedCoreRuntime) -> ProjectedCoreRuntime:
    """Fill the r x r cores of the fused apply out = a V + U (G (U^T V)),
    formed in FP64 from the factorisations:
        M^{-1}:    G = (dI + C)^{-1} - d^{-1} I,             a = 1/d
        M^{-1/2}:  G = Q diag(e^{-1/2}) Q^T - d^{-1/2} I,    a = d^{-1/2}
    (the latter only with the eigendecomposition)."""
    dd = float(rt.d)
    r = rt.total_rank
    eye64 = torch.eye(r, dtype=torch.float64, device=rt.chol.device)
    rt.a_inv = 1.0 / dd
    rt.core_inv = (torch.cholesky_inverse(rt.chol.double()) - eye64 / dd).float().contiguous()
    if rt.eigvals is not None and rt.eigvecs is not None:
        q = rt.eigvecs.double()
        rt.a_invsqrt = dd ** -0.5
        rt.core_invsqrt = ((q / torch.sqrt(rt.eigvals.double())[None, :]) @ q.T -
                           eye64 * dd ** -0.5).float().contiguous()
    return rt


def make_projected_core_precond_from_runtime(runtime) -> Optional[Callable]:
    if runtime is None:
        return None

    def apply(v):
        if runtime.core_inv is not None and isinstance(v, torch.Tensor) and v.is_cuda:
            return _lowrank_apply(v, runtime.U, runtime.core_inv, runtime.a_inv)
        return _apply_scalar_diag(v, runtime.d_inv, runtime.chol, runtime.U)

    return apply


def projected_core_apply_invsqrt(runtime: ProjectedCoreRuntime, v):
    if runtime.eigvals is None or runtime.eigvecs is None:
        raise ValueError(
            "Projected-core runtime missing eigendecomposition required for inverse-square-root apply."
        )
    if runtime.core_invsqrt is not None and isinstance(v, torch.Tensor) and v.is_cuda:
        return _lowrank_apply(v, runtime.U, runtime.core_invsqrt, runtime.a_invsqrt)
    return _apply_invsqrt(v, torch.sqrt(runtime.d_inv), runtime.eigvals, runtime.eigvecs,
                          runtime.U)


def projected_core_logdet(runtime: ProjectedCoreRuntime, n_dim: int) -> torch.Tensor:
    """(n - r) log d + 2 sum log diag(chol)  (precond.py:207-221)."""
    if n_dim < runtime.total_rank:
        raise ValueError(
            f"n_dim={n_dim} is smaller than projected-core rank {runtime.total_rank}."
        )
    cd = torch.diagonal(runtime.chol)
    tiny = torch.finfo(cd.dtype).tiny
    return (n_dim - runtime.total_rank) * torch.log(runtime.d) + 2.0 * torch.sum(
        torch.log(torch.clamp(cd, min=tiny)))


def make_projected_core_precond(precond_conf, theta_g, diag_H, eps: float = 0.0):
    runtime = build_projected_core_runtime(precond_conf, theta_g, diag_H, eps=eps,
                                           need_invsqrt=False)
    return make_projected_core_precond_from_runtime(runtime)


def make_precond(precond_conf, theta_g, diag_H, eps: float = 0.0):
    return make_projected_core_precond(precond_conf, theta_g, diag_H, eps=eps)


def build_lowrank_basis(K_mv: Callable, n: int, max_rank: int, key=0, oversample: int = 8,
                        dtype=torch.float32, device=None, omega: torch.Tensor | None = None):
    """Nystrom sketch: U, eigenvalues of the leading spectrum (precond.py:251-276).

    ``key`` seeds a torch generator for the Gaussian test matrix (the
    reference draws it from jax.random); ``omega`` may supply it directly.
    """
    r = int(max_rank) + int(oversample)
    if omega is None:
        gen = torch.Generator(device="cpu")
        gen.manual_seed(int(key))
        omega = torch.randn((n, r), generator=gen, dtype=torch.float32)
    dev = device if device is not None else (omega.device if omega.is_cuda else torch.device("cuda"))
    Omega = omega.to(device=dev, dtype=dtype)
    Y = K_mv(Omega)
    Q, _ = torch.linalg.qr(Y, mode="reduced")
    Q = Q.contiguous()
    Z = K_mv(Q)
    B = Q.T @ Z
    evals, evecs = torch.linalg.eigh(B)
    idx = torch.argsort(evals, descending=True)
    evals = torch.clamp(evals[idx], min=0.0)
    evecs = evecs[:, idx]
    U_full = Q @ evecs
    k = min(int(max_rank), U_full.shape[1])
    return U_full[:, :k].contiguous(), evals[:k]


__all__ = [
    "ProjectedCorePrecondConf",
    "ProjectedCoreRuntime",
    "build_projected_core_runtime",
    "make_projected_core_precond",
    "make_projected_core_precond_from_runtime",
    "make_precond",
    "projected_core_apply_invsqrt",
    "projected_core_logdet",
    "scalar_diag_from_precond_conf",
    "build_lowrank_basis",
]
