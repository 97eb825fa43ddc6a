"""GPU block PCG: the reference's PCG checks (tests/test_pcg_stability.py) plus
parity with the oracle on a genotype operator."""
import numpy as np
import pytest
import torch

from coherit_gb300 import pcg as gpcg
from oracle import pcg as opcg

pytestmark = pytest.mark.gpu


def _true_relative(hv, x, b):
    residual = (b - hv(x)).double().cpu().numpy()
    rhs = b.double().cpu().numpy()
    if residual.ndim == 1:
        residual, rhs = residual[:, None], rhs[:, None]
    den = np.linalg.norm(rhs, axis=0)
    return float(np.max(np.linalg.norm(residual, axis=0) / np.where(den > 0, den, 1)))


def T(a, dev):
    return torch.as_tensor(np.array(a, np.float32), device=dev)


@pytest.mark.parametrize("check_every", [1, 2, 5])
@pytest.mark.parametrize("preconditioned", [False, True])
def test_diagonal_zero_and_extreme_scales(cuda, check_every, preconditioned):
    scales = np.asarray([0, 1e-30, 1e-8, 1, 1e30], dtype=np.float32)
    b = T(np.arange(1, 17, dtype=np.float32)[:, None] * scales, cuda)
    calls = []

    def hv(v):
        calls.append(None)
        return 2 * v

    pre = (lambda v: v / 2) if preconditioned else None
    x, rel, it = gpcg.pcg_solve(hv, b, M=pre, tol=1e-6, maxiter=20, check_every=check_every)
    assert len(calls) == it + 2
    xs = x.cpu().numpy()
    np.testing.assert_allclose(xs[:, 1:] / scales[1:],
                               np.broadcast_to(np.arange(1, 17)[:, None] / 2, (16, 4)), rtol=1e-6)
    np.testing.assert_array_equal(xs[:, 0], 0)
    assert float(rel) == pytest.approx(_true_relative(hv, x, b), abs=1e-8)
    assert float(rel) <= 1e-6
    assert it <= check_every


@pytest.mark.parametrize("preconditioned", [False, True])
def test_spd_dense_with_warm_start(cuda, preconditioned):
    rng = np.random.default_rng(237)
    root = rng.normal(size=(24, 24))
    h = (root @ root.T / 24 + np.eye(24)).astype(np.float32)
    rhs = rng.normal(size=(24, 3)).astype(np.float32)
    scales = np.asarray([1e-20, 1, 1e20], dtype=np.float32)
    b = T(rhs * scales, cuda)
    hd = torch.as_tensor(h.astype(np.float64), device=cuda)
    hv = lambda v: (hd @ v.double()).float()
    diag = T(np.diag(h), cuda)
    pre = (lambda v: v / diag[:, None]) if preconditioned else None
    x, rel, _ = gpcg.pcg_solve(hv, b, M=pre, X0=0.1 * b, tol=1e-6, maxiter=100)
    expected = np.linalg.solve(h.astype(np.float64), rhs)
    np.testing.assert_allclose(x.cpu().numpy() / scales, expected, atol=2e-6, rtol=2e-5)
    assert float(rel) <= 1e-6
    assert float(rel) == pytest.approx(_true_relative(hv, x, b), rel=2e-6, abs=1e-12)


def test_vector_converged_warm_start_preserved(cuda):
    d = torch.arange(1, 9, dtype=torch.float32, device=cuda)
    hv = lambda v: d * v
    b = torch.arange(8, dtype=torch.float32, device=cuda) * 1e-20
    x0 = b / d
    x, rel, it = gpcg.pcg_solve(hv, b, X0=x0, tol=1e-6)
    assert x.shape == b.shape
    assert torch.equal(x, x0)
    assert it == 0


def test_zero_rhs_and_identity_alias(cuda):
    b = T([[0, 1], [0, -2], [0, 3]], cuda)
    x, rel, _ = gpcg.pcg_solve(lambda v: v, b, X0=torch.ones_like(b), tol=1e-6)
    assert torch.equal(x, b)
    assert float(rel) == 0


@pytest.mark.parametrize("maxiter", [1, 314])
def test_true_residual_at_budget(cuda, maxiter):
    rng = np.random.default_rng(12)
    basis = np.linalg.qr(rng.normal(size=(60, 60)))[0]
    h = (basis * np.geomspace(1, 1e4, 60)) @ basis.T
    hd = torch.as_tensor(h, device=cuda)
    b = T(rng.normal(size=(60, 2)), cuda)
    hv = lambda v: (hd @ v.double()).float()
    x, rel, it = gpcg.pcg_solve(hv, b, tol=1e-5, maxiter=maxiter)
    assert it <= maxiter
    assert float(rel) == pytest.approx(_true_relative(hv, x, b), rel=2e-6, abs=1e-10)


@pytest.mark.parametrize("maxiter", [1, 100])
def test_optimistic_recurrence_restarts(cuda, monkeypatch, maxiter):
    original = gpcg._pcg_state_update
    calls = {"updates": 0, "operator": 0}

    def lose_once(*args):
        x, r, bd = original(*args)
        calls["updates"] += 1
        if calls["updates"] == 1:
            r.zero_()
        return x, r, bd

    d = torch.linspace(1, 4, 20, device=cuda)[:, None]
    b = torch.ones((20, 1), device=cuda)

    def hv(v):
        calls["operator"] += 1
        return d * v

    monkeypatch.setattr(gpcg, "_pcg_state_update", lose_once)
    x, rel, it = gpcg.pcg_solve(hv, b, tol=1e-6, maxiter=maxiter, check_every=1)
    assert float(rel) == pytest.approx(_true_relative(hv, x, b), rel=2e-6, abs=1e-10)
    assert it <= maxiter
    if maxiter == 1:
        assert float(rel) > 1e-6
    else:
        assert calls["operator"] > it + 2
        assert float(rel) <= 1e-6
        np.testing.assert_allclose(x.cpu().numpy(), (b / d).cpu().numpy(), rtol=3e-6)


def test_zero_budget(cuda):
    b = torch.ones((5, 2), device=cuda) * 1e-20
    x, rel, it = gpcg.pcg_solve(lambda v: 2 * v, b, maxiter=0)
    assert torch.all(x == 0)
    assert it == 0
    assert float(rel) == pytest.approx(1)


@pytest.mark.parametrize("factor", [0.0, -1.0, float("nan")])
def test_invalid_operator_raises(cuda, factor):
    with pytest.raises(FloatingPointError):
        gpcg.pcg_solve(lambda v: factor * v, torch.ones((8, 1), device=cuda), maxiter=4)


def test_genotype_operator_solve_matches_oracle(cuda):
    from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
    from oracle import geno as og

    n, m = 700, 2000
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=31), precision="bf16x3")
    codes = og.synth_codes(31, n, np.arange(m))
    mean, inv = st._means_host, st._inv_sds_host
    eff = float(st._eff_m_const)
    theta_g, theta_e = 0.6, 0.4
    rng = np.random.default_rng(8)
    B = rng.normal(size=(n, 4)).astype(np.float32)

    def hv_gpu(v):
        return st.weighted_component_hv([theta_g], theta_e, v)

    def hv_cpu(v):
        return og.kv_f64(codes, mean, inv, v, comp_scale=[theta_g / eff], theta_e=theta_e).astype(np.float32)

    x, rel, it = gpcg.pcg_solve(hv_gpu, T(B, cuda), tol=1e-6, maxiter=300)
    xo, relo, ito = opcg.pcg_solve(hv_cpu, B, tol=1e-6, maxiter=300)
    assert float(rel) <= 1e-6 and relo <= 1e-6
    # Dense FP64 solve of the same system
    Z = og.diff_f64(codes, mean) * inv.astype(np.float64)
    H = theta_g * (Z @ Z.T) / eff + theta_e * np.eye(n)
    exact = np.linalg.solve(H, B.astype(np.float64))
    xs = x.cpu().numpy()
    rel_err = np.linalg.norm(xs - exact, axis=0) / np.linalg.norm(exact, axis=0)
    assert np.max(rel_err) < 1e-5
    assert abs(it - ito) <= 2


def test_lowrank_apply_matches_fp64_formulas(cuda):
    """The fused projected-core applies (coherit_lowrank_apply) against the
    explicit formulas in FP64 (precond.py:42-84): M^{-1} V and M^{-1/2} V for
    an orthonormal basis, odd n and k (partial tiles), vector and block."""
    from coherit_gb300 import precond as pc

    n, r, k = 5003, 72, 13
    g = torch.Generator(device="cpu").manual_seed(4)
    U, _ = torch.linalg.qr(torch.randn(n, r, generator=g, dtype=torch.float64))
    A = torch.randn(r, r, generator=g, dtype=torch.float64)
    C = A @ A.T / r
    d = 0.7
    U32 = U.float().contiguous().to(cuda)
    eye = torch.eye(r, dtype=torch.float32, device=cuda)
    conf = pc.ProjectedCorePrecondConf(
        U=U32, core_atoms=C.float().to(cuda)[None], total_rank=r, n_grm=1,
        diag_mode="scalar_identity", diag_atoms=torch.zeros(1, device=cuda),
        residual_diag_atoms=torch.ones(1, device=cuda), identity=eye)
    rt = pc.build_projected_core_runtime(conf, torch.ones(1, device=cuda),
                                         torch.tensor(d, device=cuda), need_invsqrt=True)
    assert rt.core_inv is not None and rt.core_invsqrt is not None
    V = torch.randn(n, k, generator=g, dtype=torch.float64)
    mid = C + d * torch.eye(r, dtype=torch.float64)
    want = V / d + U @ ((torch.linalg.inv(mid) - torch.eye(r, dtype=torch.float64) / d)
                        @ (U.T @ V))
    ev, q = torch.linalg.eigh(mid)
    isq = (q / torch.sqrt(ev)[None, :]) @ q.T - torch.eye(r, dtype=torch.float64) / d ** 0.5
    want_sq = V / d ** 0.5 + U @ (isq @ (U.T @ V))
    Vd = V.float().to(cuda)
    got = pc.make_projected_core_precond_from_runtime(rt)(Vd).double().cpu()
    got_sq = pc.projected_core_apply_invsqrt(rt, Vd).double().cpu()
    for a, b in ((got, want), (got_sq, want_sq)):
        rel = ((a - b).norm(dim=0) / b.norm(dim=0)).max().item()
        assert rel < 1e-5, rel
    vec = pc.make_projected_core_precond_from_runtime(rt)(Vd[:, 3]).double().cpu()
    assert ((vec - want[:, 3]).norm() / want[:, 3].norm()).item() < 1e-5
