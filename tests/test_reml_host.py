"""Host numerics of the REML driver, run on CPU tensors against the oracle.

The package's SLQ (slq.py:143-213 of the reference), affine SLQ
(reml.py:367-486), projected-core preconditioner (precond.py:42-276) and
bounded Fisher step (reml.py:979-1247) are plain torch / numpy code that runs
on whatever device its inputs live on; on the device they only see the
genotype operator through a callable.  Here they run on CPU over dense
operators, so the same known-answer checks that pin the oracle pin them too,
and each result is compared with the oracle on the same probes.

fit_reml itself runs here up to its first evaluation (set-up, probe caches,
tolerance clamp), and to completion with the evaluation replaced by an
analytic objective, where its steps must equal the oracle's fit.
"""
import types

import numpy as np
import pytest
import torch

from coherit_gb300 import precond as prec
from coherit_gb300 import reml
from coherit_gb300 import slq
from oracle import precond as oprec
from oracle import reml as oreml
from oracle import slq as oslq

CPU = torch.device("cpu")
EPS32 = float(np.finfo(np.float32).eps)
EPS64 = float(np.finfo(np.float64).eps)


# ------------------------------------------------------------------- SLQ

def _slq_problem(kind):
    # tests/test_multi_slq_score_consistency.py:19-35 of the reference
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


def _package_slq(directions, theta, depth, *, dtype=torch.float64, budget=64 * 1024 ** 2,
                 value_only=False, eps=EPS64, accept_value=None):
    D = torch.as_tensor(directions, dtype=dtype)
    t = torch.as_tensor(theta, dtype=dtype)
    A = torch.einsum("k,kij->ij", t, D)

    def mv(v):
        return A @ v

    def pullback(left, right):
        products = torch.einsum("kij,js->kis", D, left)
        return (torch.einsum("k,kns->ns", t, products),
                torch.einsum("ns,kns->k", right, products).double())

    value, grad = slq.logdet_value_and_grad(
        mv, None if value_only else pullback, 24, 0, nsamples=_PROBES.shape[1], m=depth,
        workspace_bytes=budget, dtype=dtype, accept_value=accept_value, device=CPU,
        probes=torch.as_tensor(_PROBES), eps=eps)
    return float(value), (None if grad is None else grad.numpy())


def _oracle_slq(directions, theta, depth, *, budget=64 * 1024 ** 2, eps=EPS64, itemsize=8):
    A = np.einsum("k,kij->ij", theta, directions)

    def pullback(left, right):
        products = np.einsum("kij,js->kis", directions, left)
        return np.einsum("k,kns->ns", theta, products), np.einsum("ns,kns->k", right, products)

    return oslq.logdet_value_and_grad(lambda v: A @ v, pullback, 24, _PROBES, m=depth,
                                      workspace_bytes=budget, itemsize=itemsize, eps=eps)


@pytest.mark.parametrize("kind", ["regular", "scalar", "clustered", "zero", "ill_conditioned"])
@pytest.mark.parametrize("depth", [1, 10, 30])
def test_slq_fp64_equals_oracle(kind, depth):
    d, t = _slq_problem(kind)
    value, grad = _package_slq(d, t, depth)
    ref_value, ref_grad = _oracle_slq(d, t, depth)
    np.testing.assert_allclose(value, ref_value, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(grad, ref_grad, rtol=1e-8, atol=1e-9)


# tests/test_multi_slq_score_consistency.py:54-71 of the reference
@pytest.mark.parametrize("kind", ["regular", "ill_conditioned"])
def test_slq_gradient_matches_finite_difference(kind):
    d, t = _slq_problem(kind)
    value, grad = _package_slq(d, t, 10)
    delta = 1e-6 if kind == "ill_conditioned" else 2e-5
    fd = []
    for k in range(len(t)):
        off = np.eye(len(t))[k] * delta
        fd.append((_package_slq(d, t + off, 10)[0] - _package_slq(d, t - off, 10)[0])
                  / (2 * delta))
    np.testing.assert_allclose(grad, fd, rtol=2e-3, atol=3e-3)


# tests/test_multi_slq_score_consistency.py:74-97 of the reference
@pytest.mark.parametrize("kind", ["regular", "scalar", "clustered", "zero", "ill_conditioned"])
def test_slq_full_depth_equals_dense_probe_form(kind):
    d, t = _slq_problem(kind)
    value, grad = _package_slq(d, t, 50, eps=EPS32)
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
    np.testing.assert_allclose(grad, np.einsum("ij,kij->k", gm, d), rtol=2e-3, atol=2e-3)
    vo = _package_slq(d, t, 50, value_only=True, eps=EPS32)
    assert vo[0] == value and vo[1] is None


# tests/test_multi_slq_score_consistency.py:100-107 of the reference
def test_slq_probe_batching_invariance():
    d, t = _slq_problem("regular")
    full = _package_slq(d, t, 10)
    single = _package_slq(d, t, 10, budget=1)
    np.testing.assert_allclose(single[0], full[0], atol=1e-10)
    np.testing.assert_allclose(single[1], full[1], atol=1e-9)


def test_slq_deferred_gradient_follows_accept_value():
    d, t = _slq_problem("regular")
    full = _package_slq(d, t, 10)
    rejected = _package_slq(d, t, 10, accept_value=lambda v: False)
    accepted = _package_slq(d, t, 10, accept_value=lambda v: True)
    assert rejected[0] == full[0] and rejected[1] is None
    assert accepted[0] == full[0]
    np.testing.assert_allclose(accepted[1], full[1], rtol=1e-12, atol=1e-14)


# tests/test_reml_lazy_evaluation.py:79-105 of the reference: a rejected value
# never costs a reverse pass when the batches fit the workspace, and the value
# never repeats a forward product.
@pytest.mark.parametrize("budget", [1, 50000, 1 << 20])
@pytest.mark.parametrize("accepted", [False, True])
@pytest.mark.parametrize("impl", ["package", "oracle"])
def test_slq_gate_preserves_value_and_never_repeats_forward_products(budget, accepted, impl):
    calls = {"forward": 0, "reverse": 0}
    diag = np.linspace(.3, 2., 24)
    probes = np.random.default_rng(54).choice([-1.0, 1.0], size=(24, 6))
    if impl == "package":
        matrix = torch.diag(torch.as_tensor(diag, dtype=torch.float32))

        def mv(b):
            calls["forward"] += 1
            return matrix @ b

        def pullback(left, right):
            calls["reverse"] += 1
            product = matrix @ left
            return product, torch.sum(product * right).double().reshape(1)

        def run(**kw):
            return slq.logdet_value_and_grad(mv, pullback, 24, 0, nsamples=6, m=8,
                                             workspace_bytes=budget, device=CPU,
                                             probes=torch.as_tensor(probes), **kw)
    else:
        matrix = np.diag(diag)

        def mv(b):
            calls["forward"] += 1
            return matrix @ b

        def pullback(left, right):
            calls["reverse"] += 1
            product = matrix @ left
            return product, np.asarray([np.sum(product * right)])

        def run(**kw):
            return oslq.logdet_value_and_grad(mv, pullback, 24, probes, m=8,
                                              workspace_bytes=budget, **kw)
    expected = run()
    eager = dict(calls)
    calls.update(forward=0, reverse=0)
    actual = run(accept_value=lambda value: accepted)
    assert float(actual[0]) == float(expected[0])
    assert calls["forward"] == eager["forward"]
    if accepted:
        np.testing.assert_array_equal(np.asarray(actual[1]), np.asarray(expected[1]))
        assert calls["reverse"] == eager["reverse"]
    else:
        assert actual[1] is None
        assert calls["reverse"] == (eager["reverse"] if budget == 1 else 0)


def test_slq_fp32_within_logdet_tolerance_of_oracle():
    d, t = _slq_problem("regular")
    value, grad = _package_slq(d, t, 10, dtype=torch.float32, eps=EPS32)
    ref_value, ref_grad = _oracle_slq(d, t, 10, eps=EPS32, itemsize=4)
    np.testing.assert_allclose(value, ref_value, rtol=1e-4)
    np.testing.assert_allclose(grad, ref_grad, rtol=1e-3, atol=1e-4)


def test_slq_rejects_non_finite_operator():
    d, t = _slq_problem("regular")
    with pytest.raises(FloatingPointError):
        slq.logdet_value_and_grad(lambda v: v * float("nan"), None, 24, 0, nsamples=4, m=5,
                                  dtype=torch.float64, device=CPU,
                                  probes=torch.as_tensor(_PROBES))


def test_rademacher_probes_are_signs_and_seeded():
    a = slq.rademacher(50, 7, 11, CPU)
    b = slq.rademacher(50, 7, 11, CPU)
    assert torch.equal(a, b)
    assert set(torch.unique(a).tolist()) <= {-1.0, 1.0}
    assert not torch.equal(a, slq.rademacher(50, 7, 12, CPU))


@pytest.mark.parametrize("args", [(100, 64, 30, 256 * 1024 ** 2), (5000, 128, 30, 1),
                                  (3, 9, 50, 10 ** 6), (50000, 64, 30, 2 * 1024 ** 3)])
def test_workspace_layout_equals_oracle(args):
    assert slq.workspace_layout(*args) == oslq.workspace_layout(*args)


# ------------------------------------------------------------ affine SLQ

def _affine_problem(n=12, width=20, seed=5):
    rng = np.random.default_rng(seed)
    raw = rng.normal(size=(n, width))
    K = raw @ raw.T / width + 0.08 * np.eye(n)
    z = rng.choice([-1.0, 1.0], size=(n, 6))
    return K, z


@pytest.mark.parametrize("m", [4, 12])
def test_affine_slq_equals_oracle(m):
    K, z = _affine_problem()
    n = K.shape[0]
    Kt = torch.as_tensor(K, dtype=torch.float32)
    cache = reml._build_affine_slq_cache(lambda v: Kt @ v, n, 0, nsamples=z.shape[1], m=m,
                                         probes=torch.as_tensor(z), device=CPU)
    ref = oslq.affine_cache(lambda v: K @ v, n, z, m)
    for tg, te in [(0.4, 0.6), (1.3, 0.2), (0.0, 1.0)]:
        ld, der = reml._affine_slq_logdet(cache, tg, te, return_derivatives=True)
        ref_ld, ref_der = oslq.affine_logdet(ref, tg, te)
        np.testing.assert_allclose(float(ld), ref_ld, rtol=1e-4)
        np.testing.assert_allclose(der.numpy(), ref_der, rtol=1e-3, atol=1e-4)
        assert float(reml._affine_slq_logdet(cache, tg, te)) == float(ld)


# tests/test_affine_slq_score_consistency.py:149-169 of the reference
def test_affine_slq_derivatives_finite_at_zero_genetic_variance():
    rng = np.random.default_rng(20260723)
    n = 10
    raw = rng.normal(size=(n, 14))
    K = torch.as_tensor(raw @ raw.T / raw.shape[1] + 0.08 * np.eye(n), dtype=torch.float32)
    z = torch.as_tensor(rng.choice([-1.0, 1.0], size=(n, 5)))
    cache = reml._build_affine_slq_cache(lambda v: K @ v, n, 0, nsamples=5, m=n, probes=z,
                                         device=CPU)
    ld, der = reml._affine_slq_logdet(cache, 0.0, 1.0, return_derivatives=True)
    assert np.isfinite(float(ld)) and bool(torch.all(torch.isfinite(der)))
    eps = 2e-3
    fwd = (float(reml._affine_slq_logdet(cache, eps, 1.0)) - float(ld)) / eps
    np.testing.assert_allclose(float(der[0]), fwd, atol=2e-2, rtol=2e-2)
    np.testing.assert_allclose(float(der[1]), n, atol=2e-4, rtol=2e-5)


# ------------------------------------------------------ projected core

def _precond_problem(n=40, r=6, G=2, seed=3):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.normal(size=(n, r)))
    atoms = []
    for _ in range(G):
        a = rng.normal(size=(r, r))
        atoms.append(a @ a.T / r)
    return U, np.stack(atoms)


def _confs(U, atoms, diag_atoms, residual_atoms):
    G, r = atoms.shape[0], U.shape[1]
    conf = prec.ProjectedCorePrecondConf(
        U=torch.as_tensor(U), core_atoms=torch.as_tensor(atoms), total_rank=r, n_grm=G,
        diag_mode="scalar_identity", diag_atoms=torch.as_tensor(diag_atoms),
        residual_diag_atoms=torch.as_tensor(residual_atoms))
    oconf = oprec.Conf(U=U, core_atoms=atoms, total_rank=r, n_grm=G, diag_atoms=diag_atoms,
                       residual_diag_atoms=residual_atoms)
    return conf, oconf


def test_projected_core_equals_oracle():
    U, atoms = _precond_problem()
    conf, oconf = _confs(U, atoms, np.array([0.9, 1.1]), np.array([1.0, 0.5]))
    theta_g, theta_e = np.array([0.3, 0.7]), np.array([0.4, 0.2])
    d = prec.scalar_diag_from_precond_conf(conf, torch.as_tensor(theta_g), theta_e)
    od = oprec.scalar_diag(oconf, theta_g, theta_e)
    assert float(d) == pytest.approx(od, rel=1e-14)
    rt = prec.build_projected_core_runtime(conf, theta_g, d, eps=1e-3, need_invsqrt=True)
    ort = oprec.runtime(oconf, theta_g, od, eps=1e-3, need_invsqrt=True)
    v = np.random.default_rng(8).normal(size=(U.shape[0], 3))
    apply = prec.make_projected_core_precond_from_runtime(rt)
    np.testing.assert_allclose(apply(torch.as_tensor(v)).numpy(), oprec.apply_inverse(ort, v),
                               rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(apply(torch.as_tensor(v[:, 0])).numpy(),
                               oprec.apply_inverse(ort, v[:, 0]), rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(prec.projected_core_apply_invsqrt(rt, torch.as_tensor(v)).numpy(),
                               oprec.apply_invsqrt(ort, v), rtol=1e-12, atol=1e-13)
    n = U.shape[0]
    assert float(prec.projected_core_logdet(rt, n)) == pytest.approx(oprec.logdet(ort, n),
                                                                     rel=1e-13)
    # M = d I + U C U^T: the inverse inverts it and the inverse square root squares to it.
    C = np.tensordot(theta_g, atoms, axes=1)
    M = float(rt.d) * np.eye(n) + U @ C @ U.T
    np.testing.assert_allclose(M @ apply(torch.as_tensor(v)).numpy(), v, atol=1e-11)
    half = prec.projected_core_apply_invsqrt(rt, torch.as_tensor(np.eye(n))).numpy()
    np.testing.assert_allclose(half @ half @ M, np.eye(n), atol=1e-10)
    np.testing.assert_allclose(float(prec.projected_core_logdet(rt, n)),
                               np.linalg.slogdet(M)[1], rtol=1e-12)


def test_projected_core_contract_errors():
    U, atoms = _precond_problem()
    conf, _ = _confs(U, atoms, np.array([1.0, 1.0]), np.array([1.0, 1.0, 1.0]))
    with pytest.raises(ValueError, match="residual_diag_atoms"):
        prec.scalar_diag_from_precond_conf(conf, torch.as_tensor([0.3, 0.7]), [0.4, 0.2])
    conf.diag_mode = None
    assert prec.scalar_diag_from_precond_conf(conf, torch.as_tensor([0.3, 0.7]), [0.4]) is None
    with pytest.raises(NotImplementedError):
        prec.build_projected_core_runtime(conf, [0.3, 0.7], 1.0)
    conf.diag_mode = "scalar_identity"
    with pytest.raises(ValueError, match="scalar diagonal"):
        prec.build_projected_core_runtime(conf, [0.3, 0.7], [1.0, 2.0])
    rt = prec.build_projected_core_runtime(conf, [0.3, 0.7], 1.0)
    with pytest.raises(ValueError, match="eigendecomposition"):
        prec.projected_core_apply_invsqrt(rt, torch.ones(U.shape[0]))
    with pytest.raises(ValueError, match="smaller than"):
        prec.projected_core_logdet(rt, U.shape[1] - 1)
    assert prec.build_projected_core_runtime(None, [0.3], 1.0) is None
    assert prec.make_precond(None, [0.3], 1.0) is None


def test_lowrank_basis_equals_oracle():
    rng = np.random.default_rng(12)
    n, width = 60, 9
    raw = rng.normal(size=(n, width))
    K = raw @ raw.T / width
    omega = rng.normal(size=(n, 7 + 4))
    Kt = torch.as_tensor(K)
    U, ev = prec.build_lowrank_basis(lambda v: Kt @ v, n, 7, oversample=4, dtype=torch.float64,
                                     device=CPU, omega=torch.as_tensor(omega))
    oU, oev = oprec.lowrank_basis(lambda v: K @ v, omega, 7)
    np.testing.assert_allclose(ev.numpy(), oev, rtol=1e-10, atol=1e-12)
    # Eigenvectors are defined up to sign: compare the projectors.
    np.testing.assert_allclose(U.numpy() @ U.numpy().T, oU @ oU.T, atol=1e-9)
    np.testing.assert_allclose(U.numpy().T @ U.numpy(), np.eye(7), atol=1e-12)
    # A rank-9 kernel sketched with 11 columns recovers its leading spectrum.
    np.testing.assert_allclose(ev.numpy(), np.linalg.eigvalsh(K)[::-1][:7], rtol=1e-8)


# ------------------------------------------------------- Fisher step

def _fisher_cases():
    rng = np.random.default_rng(2026)
    cases = []
    for G in (1, 2, 4, 8):
        for case in range(6):
            P = G + 1
            a = rng.normal(size=(P, P))
            ai = a @ a.T / P + 0.05 * np.eye(P)
            param = np.abs(rng.normal(size=P)) * 0.5
            grad = rng.normal(size=P)
            if case >= 2:
                param[: G // 2 + 1] = 0.0          # genetic components at their bound
            if case >= 3:
                grad[0] = -abs(grad[0])            # pushing further into the bound: frozen
            if case >= 4:
                param[G] = 1e-2                    # residual at its floor
                grad[G] = -abs(grad[G])
            if case == 5:
                ai = np.outer(a[0], a[0])          # rank-one: needs the ridge and jitter
            cases.append((G, param, grad, ai))
    return cases


@pytest.mark.parametrize("alpha", [1.0, 0.5, 0.25])
def test_fisher_step_equals_oracle(alpha):
    for G, param, grad, ai in _fisher_cases():
        FI = reml.AverageInfoMatrix(mat=ai)
        d, frozen = reml._projected_fisher_direction(param, grad, FI, n_genetic=G,
                                                     genetic_zero_tol=1e-8, residual_floor=1e-2,
                                                     trial_alpha=alpha)
        od = oreml.fisher_step(param, grad, ai, G=G, zero_tol=1e-8, floor=1e-2, alpha=alpha)
        np.testing.assert_allclose(d, od, rtol=1e-9, atol=1e-10)
        new, delta = reml._apply_projected_step(param, d, alpha, n_genetic=G,
                                                genetic_zero_tol=1e-8, residual_floor=1e-2)
        onew = oreml.apply_step(param, od, alpha, G=G, zero_tol=1e-8, floor=1e-2)
        np.testing.assert_allclose(new, onew, rtol=1e-9, atol=1e-10)
        np.testing.assert_allclose(delta, new - param)
        assert np.all(new[:G] >= 0) and np.all(new[G:] >= 1e-2)
        assert frozen.shape == (G,)


def test_fisher_step_is_kkt_point_of_the_bounded_qp():
    for G, param, grad, ai in _fisher_cases():
        FI = reml.AverageInfoMatrix(mat=ai)
        d, _ = reml._projected_fisher_direction(param, grad, FI, n_genetic=G,
                                                genetic_zero_tol=1e-8, residual_floor=1e-2)
        lower = np.concatenate([np.zeros(G), np.full(param.size - G, 1e-2)]) - param
        system = 0.5 * (ai + ai.T) + reml.FI_SYSTEM_RIDGE * np.eye(param.size)
        kkt = grad - system @ d
        at_bound = d <= lower + 1e-10
        tol = 1e-6 * max(1.0, np.max(np.abs(grad))) * 10
        assert np.all(d >= lower - 1e-10)
        np.testing.assert_allclose(kkt[~at_bound], 0.0, atol=tol)
        assert np.all(kkt[at_bound] <= tol)


def test_fisher_step_contract_errors():
    FI = reml.AverageInfoMatrix(mat=np.eye(3))
    with pytest.raises(ValueError):
        reml._projected_fisher_direction([1, 1, 1], [0, 0, 0], FI, n_genetic=4,
                                         genetic_zero_tol=1e-8)
    with pytest.raises(ValueError):
        reml._projected_fisher_direction([1, 1, 1], [0, 0, 0], FI, genetic_zero_tol=1e-8,
                                         residual_floor=-1.0)
    with pytest.raises(ValueError):
        reml._projected_fisher_direction([1, 1, 1], [0, 0, 0], FI, genetic_zero_tol=1e-8,
                                         trial_alpha=0.0)
    with pytest.raises(ValueError, match="shape"):
        reml._projected_fisher_direction([1, 1], [0, 0], FI, genetic_zero_tol=1e-8)
    with pytest.raises(FloatingPointError):
        reml._projected_fisher_direction([1, 1, 1], [0, np.nan, 0], FI, genetic_zero_tol=1e-8)


def test_fisher_stats_record_the_active_set():
    stats = reml.FisherSolveStats()
    FI = reml.AverageInfoMatrix(mat=np.eye(3), stats=stats)
    d, frozen = reml._projected_fisher_direction([0.0, 0.5, 0.3], [-1.0, 0.2, 0.1], FI,
                                                 genetic_zero_tol=1e-8, residual_floor=1e-2)
    assert frozen.tolist() == [True, False]
    assert d[0] == 0.0
    assert stats.frozen_genetic == 1 and stats.free_dim == 2


# ------------------------------------------------- small host helpers

def test_standardize_response_equals_oracle():
    y = np.random.default_rng(4).normal(3.0, 2.5, size=513).astype(np.float32)
    ys, mu, scale = reml.standardize_response(y)
    oys, omu, oscale = oreml.standardize(y)
    np.testing.assert_allclose(ys.numpy(), oys, rtol=1e-6, atol=1e-6)
    assert float(mu) == pytest.approx(omu, rel=1e-6)
    assert float(scale) == pytest.approx(oscale, rel=1e-6)
    for bad in ([], [1.0, float("nan")], [2.0, 2.0, 2.0]):
        with pytest.raises(ValueError):
            reml.standardize_response(np.asarray(bad, np.float32))


def test_stable_cholesky_equals_oracle():
    rng = np.random.default_rng(6)
    a = rng.normal(size=(5, 3))
    for A in (a @ a.T, a @ a.T + np.eye(5), np.diag([1.0, 1e-14, 2.0])):
        L = reml._stable_cho_factor_spd(torch.as_tensor(A)).numpy()
        np.testing.assert_allclose(L, oreml.stable_chol(A), rtol=1e-10, atol=1e-12)
    # The jitter grows to 10 x the mean |diagonal| (1 when that is 0): -I is
    # rescued, an indefinite matrix with eigenvalues +-100 and zero diagonal is not.
    np.testing.assert_allclose(reml._stable_cho_factor_spd(torch.as_tensor(-np.eye(3))).numpy(),
                               oreml.stable_chol(-np.eye(3)), rtol=1e-12)
    indefinite = np.array([[0.0, 100.0], [100.0, 0.0]])
    for fn in (lambda: reml._stable_cho_factor_spd(torch.as_tensor(indefinite)),
               lambda: oreml.stable_chol(indefinite)):
        with pytest.raises(FloatingPointError):
            fn()


def test_fixed_effect_design_validation():
    rng = np.random.default_rng(7)
    X = np.column_stack([np.ones(50), rng.normal(size=50)])
    reml._validate_fixed_effect_design(torch.as_tensor(X))
    for bad in (np.column_stack([X, np.zeros(50)]), np.column_stack([X, 2 * X[:, 1]])):
        with pytest.raises(ValueError):
            reml._validate_fixed_effect_design(torch.as_tensor(bad))


def test_mean_diag_atoms():
    atoms = reml._mean_diag_atoms([1.5, np.array([1.0, 3.0]), torch.tensor(2.0)], n_samples=2)
    np.testing.assert_array_equal(atoms, [1.5, 2.0, 2.0])
    with pytest.raises(ValueError, match="length mismatch"):
        reml._mean_diag_atoms([np.ones(3)], n_samples=2)
    with pytest.raises(ValueError):
        reml._mean_diag_atoms([np.array([-1.0, 1.0])])


# ------------------------------------------- fit_reml up to its first evaluation
#
# fit_reml's validation, probe set-up, affine SLQ cache and right-hand-side
# assembly run on the device of its inputs; the first device-bound step is
# the first _eval_once (PCG on the genotype operator).  Replacing it with a
# recorder that stops the fit checks that set-up on CPU.

class _Stop(Exception):
    pass


def _record_first_eval(monkeypatch):
    seen = []

    def recorder(ctx, pvec, warm_all, warm_ai=None, **kw):
        seen.append((ctx, np.array(pvec), kw))
        raise _Stop

    monkeypatch.setattr(reml, "_eval_once", recorder)
    return seen


def _kernels(groups):
    d, _ = _slq_problem("regular")
    mats = [torch.as_tensor(k, dtype=torch.float32) for k in d[:groups]]
    return tuple(lambda b, k=k: k @ b for k in mats), tuple(torch.diagonal(k) for k in mats)


# tests/test_multi_slq_score_consistency.py:110-137 of the reference
@pytest.mark.parametrize("groups,optimizer,requested,residual,expected", [
    (2, "strict", .005, False, 1e-5),
    (2, "strict", 1e-6, False, 1e-6),
    (1, "strict", .005, False, .005),
    (1, "strict", .005, True, 1e-5),
    (2, "smile_scoring", .005, False, .005),
])
def test_pcg_tolerance_clamp(monkeypatch, groups, optimizer, requested, residual, expected):
    seen = _record_first_eval(monkeypatch)
    K_mvs, diags = _kernels(groups)
    y = np.random.default_rng(41).normal(size=24).astype(np.float32)
    with pytest.raises(_Stop):
        reml.fit_reml(y, K_mvs, diags, None, n_rand_vec=3, maxiter=100, minq_iter=0,
                      slq_samples=3, slq_m=8, pcg_tol=requested, optimizer=optimizer,
                      verbose=False, device="cpu",
                      residual_diag_list=[torch.linspace(.5, 1.5, 24)] if residual else None)
    assert [kw["minq_tol"] for _, _, kw in seen] == [expected]


# tests/test_reml_lazy_evaluation.py:35-77 of the reference: strict fits carry
# no Hutchinson probes in their right-hand sides; scoring fits cache K_i Z for
# their probes, and switching back invalidates it.
def test_probe_columns_and_cache_follow_the_optimizer(monkeypatch):
    seen = _record_first_eval(monkeypatch)
    K_mvs, diags = _kernels(2)
    rng = np.random.default_rng(684)
    args = dict(y=rng.normal(size=24).astype(np.float32), K_mvs=K_mvs, diag_list=diags,
                covar=torch.ones((24, 1)), n_rand_vec=7, maxiter=100, minq_iter=1,
                slq_samples=4, slq_m=8, pcg_tol=1e-5, verbose=False,
                response_is_standardized=True, device="cpu")
    cache = reml.REMLProbeCache()
    with pytest.raises(_Stop):
        reml.fit_reml(**args, probe_cache=cache)
    ctx = seen[-1][0]
    assert ctx.rhs_const.shape == (24, 2) and ctx.R_rand == 0 and ctx.kvrand_stack is None
    assert cache.kvrand_stack is None
    signature = cache.signature
    with pytest.raises(_Stop):
        reml.fit_reml(**{**args, "n_rand_vec": 17}, probe_cache=cache)
    assert cache.signature == signature
    with pytest.raises(_Stop):
        reml.fit_reml(**args, optimizer="smile_scoring", probe_cache=cache)
    ctx = seen[-1][0]
    assert ctx.rhs_const.shape == (24, 9) and ctx.R_rand == 7
    assert tuple(cache.kvrand_stack.shape) == (2, 24, 7)
    probes = ctx.rhs_const[:, 2:]
    for g in range(2):
        torch.testing.assert_close(cache.kvrand_stack[g], K_mvs[g](probes))
    with pytest.raises(_Stop):
        reml.fit_reml(**args, probe_cache=cache)
    assert cache.kvrand_stack is None


def test_single_grm_affine_cache_is_reused_for_the_same_operator(monkeypatch):
    seen = _record_first_eval(monkeypatch)
    K_mvs, diags = _kernels(1)
    y = np.random.default_rng(3).normal(size=24).astype(np.float32)
    cache = reml.REMLProbeCache()
    common = dict(n_rand_vec=3, maxiter=50, slq_samples=5, slq_m=6, verbose=False,
                  device="cpu", probe_cache=cache)
    with pytest.raises(_Stop):
        reml.fit_reml(y, K_mvs, diags, None, **common)
    first = cache.affine_slq
    assert first is not None and seen[-1][0].affine_slq_cache is first
    assert tuple(first.alphas_k.shape) == (6, 5) and tuple(first.betas_k.shape) == (5, 5)
    with pytest.raises(_Stop):
        reml.fit_reml(2 * y + 1, K_mvs, diags, None, **common)
    assert cache.affine_slq is first and seen[-1][0].affine_slq_cache is first
    with pytest.raises(_Stop):        # another operator tuple: rebuilt
        reml.fit_reml(y, tuple(K_mvs), diags, None, **{**common, "seed": 1})
    assert cache.affine_slq is not first


def test_initial_parameters_and_standardisation(monkeypatch):
    seen = _record_first_eval(monkeypatch)
    K_mvs, diags = _kernels(2)
    y = np.random.default_rng(8).normal(2.0, 3.0, size=24).astype(np.float32)
    with pytest.raises(_Stop):
        reml.fit_reml(y, K_mvs, diags, None, n_rand_vec=3, maxiter=50, h2_init=0.4,
                      verbose=False, device="cpu")
    ctx, p0, _ = seen[-1]
    atoms = reml._mean_diag_atoms(diags, n_samples=24)
    np.testing.assert_allclose(p0, np.r_[np.full(2, 0.4 / atoms.sum()), 0.6])
    oys, _, _ = oreml.standardize(y)
    np.testing.assert_allclose(ctx.y.numpy(), oys, rtol=1e-6, atol=1e-6)
    with pytest.raises(_Stop):
        reml.fit_reml(y, K_mvs, diags, None, n_rand_vec=3, maxiter=50, verbose=False,
                      device="cpu", param_init=[-1.0, 1e-9 / 2, 1e-3])
    np.testing.assert_array_equal(seen[-1][1], [0.0, 0.0, 1e-2])


@pytest.mark.parametrize("kwargs,exc", [
    (dict(n_rand_vec=0), ValueError), (dict(maxiter=0), ValueError),
    (dict(minq_iter=-1), ValueError), (dict(slq_m=0), ValueError),
    (dict(h2_init=1.5), ValueError), (dict(slq_mode="dense"), ValueError),
    (dict(residual_floor=0.0), ValueError), (dict(optimizer="newton"), ValueError),
    (dict(pcg_tol=0.0), ValueError), (dict(param_init=[1.0, 1.0]), ValueError),
    (dict(covar=np.ones((24, 24))), ValueError), (dict(covar=np.ones((23, 1))), ValueError),
    (dict(residual_diag_list=[-torch.ones(24)]), ValueError),
    (dict(mean_information=object()), NotImplementedError),
])
def test_fit_reml_contract_errors(kwargs, exc):
    K_mvs, diags = _kernels(2)
    args = dict(y=np.ones(24, np.float32) + np.arange(24, dtype=np.float32), K_mvs=K_mvs,
                diag_list=diags, covar=None, n_rand_vec=3, maxiter=50, verbose=False,
                device="cpu")
    with pytest.raises(exc):
        reml.fit_reml(**{**args, **kwargs})


# tests/test_reml_probe_cache.py:55-114 of the reference (the set-up part: the
# fits themselves need the device)
@pytest.mark.parametrize("components", [1, 2])
@pytest.mark.parametrize("optimizer", ["strict", "smile_scoring"])
def test_probe_cache_follows_seed_and_operators_not_response(monkeypatch, components,
                                                            optimizer):
    seen = _record_first_eval(monkeypatch)
    rng = np.random.default_rng(73)
    n = 12
    kernels = []
    for _ in range(components):
        x = rng.normal(size=(n, 16))
        kernels.append(torch.as_tensor(x @ x.T / 16, dtype=torch.float32))
    operators = tuple(lambda v, k=k: k @ v for k in kernels)
    calls = {"probes": 0, "lanczos": 0}

    def stacked(v):
        if v.shape[1] == 7:
            calls["probes"] += 1
        return torch.stack([op(v) for op in operators])

    original = reml._build_affine_slq_cache

    def build(*args, **kwargs):
        calls["lanczos"] += 1
        return original(*args, **kwargs)

    monkeypatch.setattr(reml, "_build_affine_slq_cache", build)
    cache = reml.REMLProbeCache()
    base = dict(K_mvs=operators, diag_list=[torch.diagonal(k) for k in kernels],
                stacked_kv=stacked, covar=torch.ones((n, 1)), n_rand_vec=7, maxiter=100,
                minq_iter=0, slq_samples=4, slq_m=8, response_is_standardized=True,
                pcg_tol=1e-5, verbose=False, optimizer=optimizer, device="cpu")
    traces = int(optimizer == "smile_scoring")
    single = int(components == 1)

    def fit(**kw):
        with pytest.raises(_Stop):
            reml.fit_reml(**{**base, **kw})
        return seen[-1][0]

    first = fit(y=rng.normal(size=n), probe_cache=cache)
    assert calls == {"probes": traces, "lanczos": single}
    theta = np.array([0.2] * components + [0.6])
    cached = fit(y=rng.normal(size=n), param_init=theta, probe_cache=cache)
    assert calls == {"probes": traces, "lanczos": single}
    assert cached.kvrand_stack is first.kvrand_stack
    assert cached.affine_slq_cache is first.affine_slq_cache
    fresh = fit(y=rng.normal(size=n), param_init=theta)
    assert calls == {"probes": 2 * traces, "lanczos": 2 * single}
    if traces:
        torch.testing.assert_close(fresh.kvrand_stack, cached.kvrand_stack)
    if single:
        torch.testing.assert_close(fresh.affine_slq_cache.alphas_k,
                                   cached.affine_slq_cache.alphas_k)
    before = dict(calls)
    fit(y=rng.normal(size=n), seed=91, probe_cache=cache)
    assert calls == {"probes": before["probes"] + traces, "lanczos": before["lanczos"] + single}
    before = dict(calls)
    previous = None if cache.kvrand_stack is None else cache.kvrand_stack.clone()
    changed = tuple(lambda v, k=k: 2 * k @ v for k in kernels)
    fit(y=rng.normal(size=n), seed=91, probe_cache=cache, K_mvs=changed, stacked_kv=None)
    if traces:
        torch.testing.assert_close(cache.kvrand_stack, 2 * previous)
    else:
        assert cache.kvrand_stack is None
    assert cache.signature[0] == changed
    assert calls["lanczos"] == before["lanczos"] + single


# -------------------------------------- the AI-REML driver on an analytic objective
#
# With the evaluation replaced by a concave quadratic log-likelihood whose AI
# matrix under-estimates its curvature (so full steps overshoot and the line
# search halves them) and whose unconstrained optimum has a negative genetic
# component (so the bound is active), the package's fit_reml and the
# oracle's fit must take the same steps (reml.py:1465-1880 of the reference).

def _quadratic(G, E=1):
    rng = np.random.default_rng(40 + G + 10 * E)
    P = G + E
    a = rng.normal(size=(P, P))
    A = a @ a.T / P + 0.5 * np.eye(P)
    star = np.abs(rng.normal(size=P)) * 0.3 + 0.05
    star[0] = -0.05                                    # outside theta_g >= 0
    ll = lambda t: -3.0 - 0.5 * (t - star) @ A @ (t - star)
    grad = lambda t: -A @ (t - star)
    return ll, grad, 0.3 * A


@pytest.mark.parametrize("G,E", [(1, 1), (2, 1), (4, 1), (1, 2), (3, 2)])
def test_driver_steps_equal_oracle_on_analytic_objective(monkeypatch, G, E):
    ll_of, grad_of, ai = _quadratic(G, E)

    def package_eval(ctx, pvec, warm_all, warm_ai=None, *, min_loglik=None, **kw):
        t = np.asarray(pvec, np.float64)
        ll = float(ll_of(t))
        if min_loglik is not None and not ll >= min_loglik:
            return (ll, None, None, 3, warm_all, None, None, None, None)
        FI = reml.AverageInfoMatrix(mat=ai.copy(), stats=reml.FisherSolveStats(ai_pcg_iters=4))
        return (ll, grad_of(t), FI, 7, warm_all, warm_ai, None, None, None)

    def oracle_eval(ctx, theta, *, warm=None, min_loglik=None, taylor=None):
        t = np.asarray(theta, np.float64)
        ll = float(ll_of(t))
        if min_loglik is not None and not ll >= min_loglik:
            return dict(ll=ll, grad=None, ai=None, sol=None, logdet=None, pcg=3)
        return dict(ll=ll, grad=grad_of(t), ai=ai.copy(), sol=None, logdet=None, pcg=7)

    monkeypatch.setattr(reml, "_eval_once", package_eval)
    monkeypatch.setattr(oreml, "evaluate", oracle_eval)
    K_mvs, _ = _kernels(min(G, 3)) if G <= 3 else _kernels(3)
    K_mvs = tuple(K_mvs[g % len(K_mvs)] for g in range(G))
    atoms = np.linspace(0.8, 1.2, G)
    diags = [torch.tensor(float(a)) for a in atoms]
    y = np.random.default_rng(1).normal(size=24).astype(np.float32)
    # Residual diagonals exact in FP32, so both sides average the same values.
    R = None if E == 1 else np.stack([np.ones(24), 0.5 + np.arange(24) / 16.0])
    param, history, diag = reml.fit_reml(
        y, K_mvs, diags, None, n_rand_vec=3, maxiter=50, minq_iter=30, slq_samples=3, slq_m=4,
        verbose=False, device="cpu", return_diagnostics=True,
        residual_diag_list=None if R is None else [torch.as_tensor(r) for r in R])
    # The reference averages the kernel diagonals in FP32 (reml.py:187-212).
    ctx = types.SimpleNamespace(G=G, E=E, R=R,
                                diag_atoms=atoms.astype(np.float32).astype(np.float64))
    oparam, ohist, _ = oreml.fit(ctx, minq_iter=30)
    assert len(history) == len(ohist)
    for h, o in zip(history, ohist):
        assert h["accepted"] == o["accepted"]
        np.testing.assert_allclose(h["params"], o["params"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(param, oparam, rtol=1e-12, atol=1e-14)
    assert any(h["step_alpha"] < 1.0 for h in history)      # the line search halved
    assert param[0] == 0.0                                    # the bound is active
    last = history[-1]
    assert last["stop_reason"] in ("rel_dll", "ll_down", "max_iter")
    for key in ("step_norm", "step_sec", "eval_ai_pcg_iters", "eval_sec", "free_dim",
                "frozen_genetic", "ai_pcg_iters", "ws_trace"):
        assert key in last, key
    assert diag["loglik"] == pytest.approx(ll_of(param))


def test_preconditioner_refresh_follows_accepted_non_final_steps(monkeypatch):
    """reml.py:1922-1940 of the reference: after an accepted step that does not
    end the fit (and is not the last allowed iteration) the PCG
    preconditioner is rebuilt at the accepted parameters."""
    ll_of, grad_of, ai = _quadratic(2, 1)
    seen_conf = []

    def package_eval(ctx, pvec, warm_all, warm_ai=None, *, min_loglik=None, **kw):
        seen_conf.append(ctx.precond_conf)
        t = np.asarray(pvec, np.float64)
        ll = float(ll_of(t))
        if min_loglik is not None and not ll >= min_loglik:
            return (ll, None, None, 3, warm_all, None, None, None, None)
        FI = reml.AverageInfoMatrix(mat=ai.copy(), stats=reml.FisherSolveStats(ai_pcg_iters=4))
        return (ll, grad_of(t), FI, 7, warm_all, warm_ai, None, None, None)

    monkeypatch.setattr(reml, "_eval_once", package_eval)
    refreshes = []

    def refresh(theta):
        refreshes.append(np.array(theta))
        return ("conf", len(refreshes))

    K_mvs, _ = _kernels(2)
    diags = [torch.tensor(0.9), torch.tensor(1.1)]
    y = np.random.default_rng(1).normal(size=24).astype(np.float32)
    args = (y, K_mvs, diags, None)
    kw = dict(n_rand_vec=3, maxiter=50, minq_iter=30, slq_samples=3, slq_m=4, verbose=False,
              device="cpu")
    param, hist = reml.fit_reml(*args, **kw, precond_refresh_fn=refresh)
    flagged = [h for h in hist if h["pcg_precond_refreshed"]]
    assert len(flagged) == len(refreshes) == sum(
        1 for h in hist if h["accepted"] and not h["converged"])
    for h, theta in zip(flagged, refreshes):
        np.testing.assert_array_equal(h["params"], theta)
    # The evaluations after a refresh see the rebuilt configuration.
    assert refreshes and ("conf", len(refreshes)) in seen_conf
    with pytest.raises(RuntimeError, match="returned no configuration"):
        reml.fit_reml(*args, **kw, precond_refresh_fn=lambda theta: None)


def test_fused_cores_reproduce_the_explicit_applies():
    """The r x r cores the GPU's fused apply uses (a V + U (G (U^T V)))
    reproduce M^{-1} V and M^{-1/2} V of the explicit formulas
    (precond.py:42-84), computed here on host tensors."""
    import torch

    from coherit_gb300 import precond as pc

    g = torch.Generator().manual_seed(7)
    n, r, k = 300, 12, 5
    U, _ = torch.linalg.qr(torch.randn(n, r, generator=g, dtype=torch.float64))
    A = torch.randn(r, r, generator=g, dtype=torch.float64)
    C = (A @ A.T / r).float()
    conf = pc.ProjectedCorePrecondConf(
        U=U.float(), core_atoms=C[None], total_rank=r, n_grm=1, diag_mode="scalar_identity",
        diag_atoms=torch.zeros(1), residual_diag_atoms=torch.ones(1), identity=torch.eye(r))
    rt = pc.build_projected_core_runtime(conf, torch.ones(1), torch.tensor(0.8),
                                         need_invsqrt=True)
    assert rt.core_inv is None                       # host tensors: explicit applies
    pc.fused_cores(rt)
    V = torch.randn(n, k, generator=g)
    Uf = rt.U
    fused = rt.a_inv * V + Uf @ (rt.core_inv @ (Uf.T @ V))
    explicit = pc.make_projected_core_precond_from_runtime(rt)(V)
    torch.testing.assert_close(fused, explicit, rtol=1e-4, atol=1e-5)
    fused_sq = rt.a_invsqrt * V + Uf @ (rt.core_invsqrt @ (Uf.T @ V))
    torch.testing.assert_close(fused_sq, pc.projected_core_apply_invsqrt(rt, V),
                               rtol=1e-4, atol=1e-5)
