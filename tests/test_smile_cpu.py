"""The SMILE block-weighted operator's host logic on CPU, against the oracle.

SmileBlockWeightedOperator reaches the genotypes only through the streamer's
``standardized_columns``, ``xtv`` and ``zxb``.  A streamer that computes
those from an explicit standardised matrix on CPU runs the rest of it — block
buckets, W-weighted scores, the trace normaliser, the diagonal, weighted H V,
SNP effects, multi-GRM groups (smile_block_w.py:44-914 of the reference) —
and it must equal oracle/smile.py within 1e-5 relative per column.
"""
import numpy as np
import pytest
import torch

from coherit_gb300.smile_block_w import (SmileBlockWeightedOperator,
                                         SmileMultiBlockWeightedOperator)
from oracle import geno as og
from oracle import smile as osm

TOL = 1e-5


class _HostStreamer:
    def __init__(self, Z):
        self.Z = np.asarray(Z, np.float64)
        self.n, self.m = self.Z.shape
        self.dev = torch.device("cpu")

    def standardized_columns(self, idx):
        return torch.as_tensor(self.Z[:, np.asarray(idx)], dtype=torch.float32)

    def xtv(self, V, normalize=False):
        assert not normalize
        return torch.as_tensor(self.Z.T @ torch.as_tensor(V).double().numpy(),
                               dtype=torch.float32)

    def zxb(self, b):
        return torch.as_tensor(self.Z @ torch.as_tensor(b).double().numpy(), dtype=torch.float32)


def col_rel(out, ref):
    out = np.asarray(out, np.float64).reshape(len(ref), -1)
    ref = np.asarray(ref, np.float64).reshape(len(ref), -1)
    return float(np.max(np.linalg.norm(out - ref, axis=0) /
                        np.maximum(np.linalg.norm(ref, axis=0), 1e-300)))


def wishart(rng, p):
    X = rng.normal(size=(p, p))
    return (X @ X.T / p).astype(np.float32)


def _Z(n, m, seed):
    codes = og.synth_codes(seed, n, np.arange(m), missing_q24=int(0.01 * (1 << 24)))
    mean, inv, _ = og.stats(codes)
    return osm.standardized(codes, mean, inv)


@pytest.mark.parametrize("diag_mode", ["full", "mean"])
def test_operator_matches_oracle(diag_mode):
    n, m = 120, 450
    Z = _Z(n, m, 62)
    rng = np.random.default_rng(1)
    Ws = [wishart(rng, 150), wishart(rng, 210), wishart(rng, 90)]
    op = SmileBlockWeightedOperator(_HostStreamer(Z), Ws, diag_mode=diag_mode)
    ok = osm.SmileKernel(Z, [(0, Ws[0]), (150, Ws[1]), (360, Ws[2])])
    assert abs(op.normalizer - ok.c) <= 1e-6 * ok.c
    V = rng.normal(size=(n, 5)).astype(np.float32)
    assert col_rel(op.kv(V).numpy(), ok.kv(V)) < TOL
    assert col_rel(op.kv(V[:, 0]).numpy(), ok.kv(V[:, :1])) < TOL
    assert col_rel(op.block_kv(V, 1).numpy(), ok.kv(V, block_idx=1)) < TOL
    stacked = op.stacked_block_kv(V).numpy()
    assert stacked.shape == (3, n, 5) and col_rel(stacked.sum(0), ok.kv(V)) < TOL
    assert col_rel(op.weighted_hv(0.7, 0.4, V).numpy(), ok.weighted_hv(0.7, 0.4, V)) < TOL
    beta = op.snp_effects(V[:, 2], np.array([0.7])).numpy()
    assert col_rel(beta, ok.snp_effects(V[:, 2], 0.7)) < TOL
    if diag_mode == "full":
        assert col_rel(op.diag().numpy(), ok.diag_full()) < TOL
    else:
        assert abs(float(op.diag()) - ok.diag_mean()) < 1e-6
    with pytest.raises(IndexError):
        op.block_kv(V, 3)


def test_identity_blocks_and_effective_rank():
    n, m = 100, 300
    Z = _Z(n, m, 63)
    st = _HostStreamer(Z)
    op = SmileBlockWeightedOperator.identity(st, block_size=64)
    assert op.n_blocks == 5
    ok = osm.SmileKernel.identity(Z, 64)
    assert abs(op.normalizer - ok.c) <= 1e-6 * ok.c
    V = np.random.default_rng(2).normal(size=(n, 4)).astype(np.float32)
    assert col_rel(op.kv(V).numpy(), ok.kv(V)) < TOL
    assert SmileBlockWeightedOperator.identity(st, block_size=64,
                                               normalization="effective_rank").normalizer == m
    rng = np.random.default_rng(3)
    with pytest.raises(ValueError, match="effective rank"):
        SmileBlockWeightedOperator(st, [wishart(rng, 300)], normalization="effective_rank")
    ranked = SmileBlockWeightedOperator(st, [wishart(rng, 300)], normalization="effective_rank",
                                        effective_ranks=[220.0])
    assert ranked.normalizer == 220.0
    with pytest.raises(ValueError, match="cover"):
        SmileBlockWeightedOperator(st, [wishart(rng, 200)])
    with pytest.raises(ValueError, match="exceeds"):
        SmileBlockWeightedOperator(st, [wishart(rng, 200), wishart(rng, 150)])
    part = SmileBlockWeightedOperator(st, [wishart(rng, 50)], strict_coverage=False,
                                      start_offsets=[120])
    assert part.blocks[0].start == 120


def test_multi_grm_groups_match_oracle():
    n, m = 100, 400
    Z = _Z(n, m, 65)
    rng = np.random.default_rng(4)
    groups = [[wishart(rng, 150), wishart(rng, 100)], [wishart(rng, 150)]]
    mop = SmileMultiBlockWeightedOperator.from_weight_matrix_groups(_HostStreamer(Z), groups)
    assert mop.n_grm == 2
    k0 = osm.SmileKernel(Z, [(0, groups[0][0]), (150, groups[0][1])])
    k1 = osm.SmileKernel(Z, [(250, groups[1][0])])
    V = rng.normal(size=(n, 3)).astype(np.float32)
    assert col_rel(mop.kv(V, 1).numpy(), k1.kv(V)) < TOL
    stacked = mop.stacked_kv(V).numpy()
    assert col_rel(stacked[0], k0.kv(V)) < TOL and col_rel(stacked[1], k1.kv(V)) < TOL
    got = mop.weighted_hv(np.array([0.3, 1.2]), 0.5, V).numpy()
    assert col_rel(got, osm.multi_weighted_hv([k0, k1], [0.3, 1.2], 0.5, V)) < TOL
    effects = mop.snp_effects(V[:, 0], np.array([0.3, 1.2]))
    assert col_rel(effects[0].numpy(), k0.snp_effects(V[:, 0], 0.3)) < TOL
    assert col_rel(effects[1].numpy(), k1.snp_effects(V[:, 0], 1.2)) < TOL
    with pytest.raises(ValueError):
        mop.weighted_hv(np.array([0.3]), 0.5, V)


def test_smile_reml_fit_matches_oracle(monkeypatch):
    """A single SMILE-GRM REML fit with the operator's weighted H V; the
    block PCG is replaced by an exact solve (it is checked on the GPU)."""
    from coherit_gb300 import reml
    from oracle import reml as oreml
    from oracle import slq as oslq

    def dense_solve(Hv, B, M=None, tol=1e-2, maxiter=200, X0=None, check_every=2):
        B2 = torch.as_tensor(B)
        vec = B2.ndim == 1
        B2 = (B2[:, None] if vec else B2).float()
        H = torch.as_tensor(Hv(torch.eye(B2.shape[0]))).double()
        X = torch.linalg.solve(0.5 * (H + H.T), B2.double()).float()
        R = B2.double() - torch.as_tensor(Hv(X)).double()
        rel = torch.max(R.norm(dim=0) / B2.double().norm(dim=0).clamp_min(1e-300))
        return (X[:, 0] if vec else X), rel, 1

    monkeypatch.setattr(reml, "pcg_solve", dense_solve)
    n, m = 160, 600
    Z = _Z(n, m, 66)
    rng = np.random.default_rng(5)
    Ws = [wishart(rng, 200) for _ in range(3)]
    op = SmileBlockWeightedOperator(_HostStreamer(Z), Ws, diag_mode="mean")
    ok = osm.SmileKernel(Z, [(200 * i, W) for i, W in enumerate(Ws)])
    K = ok.dense()
    beta = np.zeros(m)
    beta[rng.choice(m, 40, replace=False)] = rng.normal(size=40)
    g = Z @ beta
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = (g / g.std() * np.sqrt(0.5) + rng.normal(scale=np.sqrt(0.5), size=n)).astype(np.float32)
    probes = rng.choice([-1.0, 1.0], size=(n, 16))
    param, _, d = reml.fit_reml(y, [op.kv], [op.diag()], X, n_rand_vec=4, maxiter=500,
                                minq_iter=20, slq_samples=16, slq_m=16, pcg_tol=1e-5,
                                verbose=False, weighted_hv=op.weighted_hv,
                                return_diagnostics=True, device="cpu",
                                slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    yo, _, _ = oreml.standardize(y)
    cache = oslq.affine_cache(lambda v: K @ v, n, probes, 16)
    atom = float(np.float32(ok.diag_mean()))
    ctx = oreml.Context(yo, [lambda v: K @ v], X, diag_atoms=[atom], affine_cache=cache,
                        pcg_tol=1e-6, maxiter=500)
    po, _, cur = oreml.fit(ctx, minq_iter=20)
    h2, h2o = oreml.heritability(param, 1, [atom]), oreml.heritability(po, 1, [atom])
    assert abs(h2 - h2o) < 1e-3, (h2, h2o)
    assert abs(d["loglik"] - cur["ll"]) <= 1e-4 * abs(cur["ll"])
