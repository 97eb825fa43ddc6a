"""Effect estimation and prediction (reml_model.py:1459-1818) on CPU.

The fitter reaches the genotypes through its streamers' operator methods and
solves H X = B with pcg_solve.  A streamer that computes those methods from
explicit standardised genotypes on CPU, with pcg_solve replaced by an exact
solve, runs the fitter's own assembly: GLS fixed effects, BLUP random
effects per component, SNP effects, the projected-core preconditioner
build, and prediction on a test streamer that takes the training
standardisation.  Results must equal the dense FP64 formulas within 1e-5.
The same stand-in runs fit_infinitesimal end to end against the oracle's fit.
"""
import numpy as np
import pytest
import torch

from coherit_gb300 import pcg
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter
from oracle import geno as og
from oracle import reml as oreml


class _HostGeno:
    """Dense stand-in for GenoBlockStreamer over given codes (0/1/2, 3 = missing)."""

    has_sparse_backend = False

    def __init__(self, codes, comps=None):
        self.codes = np.asarray(codes)
        self.n, self.m = self.codes.shape
        self.dev = torch.device("cpu")
        sizes = [self.m] if comps is None else list(comps)
        self.n_components = len(sizes)
        self._component_snp_offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
        self._n_calls = len(sizes)
        self._call_snp_starts = self._component_snp_offsets[:-1].copy()
        self._call_true_widths = np.asarray(sizes, np.int32)
        mean, inv, _ = og.stats(self.codes)
        self.set_standardization(mean, inv)

    def set_standardization(self, means, inv_sds):
        self._means_host = np.asarray(means, np.float32)
        self._inv_sds_host = np.asarray(inv_sds, np.float32)
        self.Z = og.diff_f64(self.codes, self._means_host) * \
            self._inv_sds_host.astype(np.float64)[None, :]
        off = self._component_snp_offsets
        self._component_eff_m_host = np.asarray(
            [np.count_nonzero(self._inv_sds_host[a:b] > 0) for a, b in zip(off[:-1], off[1:])],
            np.float32)
        self._eff_m_host = float(np.count_nonzero(self._inv_sds_host > 0))
        self._component_mean_diag_atoms_host = np.asarray(
            [np.sum(self.Z[:, a:b] ** 2) / self.n / e
             for a, b, e in zip(off[:-1], off[1:], self._component_eff_m_host)], np.float32)
        self._mean_diag_atom_host = float(np.sum(self.Z ** 2) / self.n / self._eff_m_host)

    def _Zg(self, g):
        a, b = self._component_snp_offsets[g], self._component_snp_offsets[g + 1]
        return self.Z[:, a:b]

    @staticmethod
    def _t(x):
        return torch.as_tensor(x, dtype=torch.float32)

    def kv(self, V, normalize=True, *, precision=None):
        V = torch.as_tensor(V).double().numpy()
        out = self.Z @ (self.Z.T @ V)
        return self._t(out / self._eff_m_host if normalize else out)

    def _kv_raw(self, V, *, comp_scale, precision=None, **kw):
        V = torch.as_tensor(V).double().numpy()
        return self._t(sum(float(s) * (self._Zg(g) @ (self._Zg(g).T @ V))
                           for g, s in enumerate(comp_scale)))

    def component_kv(self, V, g, normalize=True, *, precision=None):
        V = torch.as_tensor(V).double().numpy()
        Zg = self._Zg(g)
        return self._t(Zg @ (Zg.T @ V) / (self._component_eff_m_host[g] if normalize else 1.0))

    def stacked_component_kv(self, V, normalize=True, *, precision=None):
        return torch.stack([self.component_kv(V, g, normalize) for g in range(self.n_components)])

    def weighted_component_hv(self, theta_g, theta_e, V, *, precision=None):
        out = sum(float(t) * self.component_kv(V, g) for g, t in enumerate(theta_g))
        return out + (0.0 if theta_e is None else float(theta_e)) * self._t(V)

    def xtv(self, V, normalize=False, *, precision=None):
        out = self.Z.T @ torch.as_tensor(V).double().numpy()
        return self._t(out / self._eff_m_host if normalize else out)

    def zxb(self, b, *, precision=None):
        return self._t(self.Z @ torch.as_tensor(b).double().numpy())

    def diag(self):
        return torch.tensor(self._mean_diag_atom_host, dtype=torch.float32)

    def component_diag_list(self):
        return [torch.tensor(float(a)) for a in self._component_mean_diag_atoms_host]

    def build_projected_core_atoms(self, U, *, subtract_identity=True):
        U = torch.as_tensor(U).double().numpy()
        out = np.stack([U.T @ (self._Zg(g) @ (self._Zg(g).T @ U)) / self._component_eff_m_host[g]
                        for g in range(self.n_components)])
        return self._t(out - np.eye(U.shape[1]) if subtract_identity else out)


def _exact_solve(Hv, B, M=None, tol=1e-2, maxiter=200, X0=None, check_every=2):
    B2 = torch.as_tensor(B).float()
    vec = B2.ndim == 1
    B2 = B2[:, None] if vec else B2
    H = torch.as_tensor(Hv(torch.eye(B2.shape[0]))).double()
    X = torch.linalg.solve(0.5 * (H + H.T), B2.double()).float()
    R = B2.double() - torch.as_tensor(Hv(X)).double()
    rel = torch.max(R.norm(dim=0) / B2.double().norm(dim=0).clamp_min(1e-300))
    return (X[:, 0] if vec else X), rel, 1


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("comps,precond_rank", [(None, 0), (None, 16), ([300, 500], 0),
                                                ([300, 500], 12)])
def test_effects_and_prediction_match_dense(monkeypatch, comps, precond_rank):
    monkeypatch.setattr(pcg, "pcg_solve", _exact_solve)
    n_tr, n_te, m = 150, 60, 800
    codes = og.synth_codes(71, n_tr + n_te, np.arange(m), missing_q24=int(0.01 * (1 << 24)))
    st_tr, st_te = _HostGeno(codes[:n_tr], comps), _HostGeno(codes[n_tr:], comps)
    rng = np.random.default_rng(3)
    y = rng.normal(size=n_tr + n_te).astype(np.float32)
    X = np.column_stack([np.ones(n_tr + n_te), rng.normal(size=(n_tr + n_te, 2))])
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=precond_rank, effect_pcg_tol=1e-6,
                                               vc_block_sizes=comps), [st_tr])
    G = 1 if comps is None else 2
    theta = np.array([0.45, 0.55]) if G == 1 else np.array([0.3, 0.25, 0.5])
    eff = fitter.estimate_effects(y[:n_tr], var_components=theta, covar=X[:n_tr])
    # Dense FP64 formulas (reml_model.py:1543-1644).
    Zs = [st_tr._Zg(g) for g in range(G)]
    effs = [float(e) for e in st_tr._component_eff_m_host]
    Ks = [Z @ Z.T / e for Z, e in zip(Zs, effs)]
    H = sum(t * K for t, K in zip(theta[:-1], Ks)) + theta[-1] * np.eye(n_tr)
    ys, ym, ysc = oreml.standardize(y[:n_tr])
    Hy, HX = np.linalg.solve(H, ys), np.linalg.solve(H, X[:n_tr])
    fixed = np.linalg.solve(X[:n_tr].T @ HX, X[:n_tr].T @ Hy)
    alpha = Hy - HX @ fixed
    rcomps = [t * (K @ alpha) for t, K in zip(theta[:-1], Ks)]
    snps = [t / e * (Z.T @ alpha) for t, Z, e in zip(theta[:-1], Zs, effs)]
    assert rel(eff.fixed_effects, fixed) < 1e-5
    assert rel(eff.random_effect, sum(rcomps)) < 1e-5
    for g in range(G):
        assert rel(eff.random_effect_components[g], rcomps[g]) < 1e-5
        assert rel(eff.snp_effects[g], snps[g]) < 1e-5
    assert (fitter.precond_conf is not None) == (precond_rank > 0)
    test = InfinitesimalREMLFitter(FitConfig(vc_block_sizes=comps, precond_rank=0), [st_te])
    pred = fitter.predict(eff, test_fitter=test, test_covar=X[n_tr:])
    np.testing.assert_array_equal(st_te._means_host, st_tr._means_host)
    Zt = og.diff_f64(codes[n_tr:], st_tr._means_host) * st_tr._inv_sds_host.astype(np.float64)
    y_std = X[n_tr:] @ fixed + Zt @ np.concatenate(snps)
    assert rel(pred.y_pred_std, y_std) < 1e-5
    assert rel(pred.y_pred, ym + ysc * y_std) < 1e-5
    with pytest.raises(ValueError, match="covariates"):
        fitter.predict(eff, test_fitter=test, test_covar=None)
    with pytest.raises(ValueError, match="length mismatch"):
        fitter.estimate_effects(y[:n_tr], var_components=theta[:-1], covar=X[:n_tr])


@pytest.mark.parametrize("comps", [None, [300, 500]])
def test_fit_infinitesimal_matches_oracle_fit(monkeypatch, comps):
    """The model API end to end (operator bundle, projected-core
    preconditioner and its refresh, SLQ, Fisher steps), PCG replaced by an
    exact solve: |dh2| < 1e-3 against the oracle's fit."""
    from coherit_gb300 import reml
    from oracle import slq as oslq

    monkeypatch.setattr(reml, "pcg_solve", _exact_solve)
    n, m = 200, 800
    codes = og.synth_codes(81, n, np.arange(m))
    st = _HostGeno(codes, comps)
    rng = np.random.default_rng(8)
    beta = np.zeros(m)
    beta[rng.choice(m, 50, replace=False)] = rng.normal(size=50)
    g = st.Z @ beta
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = (g / g.std() * np.sqrt(0.5) + rng.normal(scale=np.sqrt(0.5), size=n)).astype(np.float32)
    probes = rng.choice([-1.0, 1.0], size=(n, 16))
    cfg = FitConfig(slq_samples=16, slq_m=16, precond_rank=12, reml_pcg_tol=1e-5, minq_iter=15,
                    slq_mode="raw", vc_block_sizes=comps, verbose=False)
    res = InfinitesimalREMLFitter(cfg, [st]).fit_infinitesimal(
        y, X, slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    G = 1 if comps is None else 2
    Zs = [st._Zg(k) for k in range(G)]
    Ks = [Z @ Z.T / float(e) for Z, e in zip(Zs, st._component_eff_m_host)]
    atoms = (np.asarray([st._mean_diag_atom_host]) if G == 1
             else st._component_mean_diag_atoms_host.astype(np.float64))
    yo, _, _ = oreml.standardize(y)
    kw = (dict(affine_cache=oslq.affine_cache(lambda v: Ks[0] @ v, n, probes, 16)) if G == 1
          else dict(slq_probes=probes, slq_m=16))
    ctx = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X, diag_atoms=atoms,
                        pcg_tol=1e-6, maxiter=1000, **kw)
    po, _, cur = oreml.fit(ctx, minq_iter=15)
    h2_ref = oreml.heritability(po, G, atoms)
    assert abs(res.heritability - h2_ref) < 1e-3, (res.heritability, h2_ref)
    assert abs(res.final_loglik - cur["ll"]) <= 1e-4 * abs(cur["ll"])
    assert res.final_ai.shape == (G + 1, G + 1) and len(res.history) >= 1


def test_dense_plus_rare_streamer_fit_matches_oracle(monkeypatch):
    """A dense GRM and a rare-variant GRM as two streamers (reml_model.py:611-666,
    :1196-1290): per-streamer operators, the summed preconditioner kernel and
    its refresh, against the oracle's two-GRM fit.  Prediction refuses
    rare-variant streamers."""
    from coherit_gb300 import reml, synth
    from oracle import sparse12 as osp

    class _Rare(_HostGeno):
        has_sparse_backend = True

    monkeypatch.setattr(reml, "pcg_solve", _exact_solve)
    n = 200
    dense = _HostGeno(og.synth_codes(91, n, np.arange(600)))
    lo, hi = synth.maf_range_q24(0.0005, 0.01)
    rare = _Rare(osp.synth_rare_codes(92, n, np.arange(900), lo, hi))
    rng = np.random.default_rng(9)
    g = dense.Z @ rng.normal(size=600) + rare.Z @ rng.normal(size=900)
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    y = (g / g.std() * np.sqrt(0.5) + rng.normal(scale=np.sqrt(0.5), size=n)).astype(np.float32)
    probes = rng.choice([-1.0, 1.0], size=(n, 16))
    cfg = FitConfig(slq_samples=16, slq_m=16, precond_rank=12, reml_pcg_tol=1e-5, minq_iter=15,
                    slq_mode="raw", verbose=False)
    fitter = InfinitesimalREMLFitter(cfg, [dense, rare])
    assert fitter._has_sparse and fitter._n_dense_streamers == 1
    res = fitter.fit_infinitesimal(y, X, slq_probes=torch.as_tensor(probes, dtype=torch.float32))
    Ks = [s.Z @ s.Z.T / s._eff_m_host for s in (dense, rare)]
    atoms = np.asarray([dense._mean_diag_atom_host, rare._mean_diag_atom_host], np.float32)
    atoms = atoms.astype(np.float64)
    yo, _, _ = oreml.standardize(y)
    ctx = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X, diag_atoms=atoms,
                        slq_probes=probes, slq_m=16, pcg_tol=1e-6, maxiter=1000)
    po, _, cur = oreml.fit(ctx, minq_iter=15)
    h2_ref = oreml.heritability(po, 2, atoms)
    assert abs(res.heritability - h2_ref) < 1e-3, (res.heritability, h2_ref)
    assert abs(res.final_loglik - cur["ll"]) <= 1e-4 * abs(cur["ll"])
    monkeypatch.setattr(pcg, "pcg_solve", _exact_solve)
    eff = fitter.estimate_effects(y, var_components=res.var_components, covar=X)
    with pytest.raises(NotImplementedError, match="dense genotype paths only"):
        fitter.predict(eff, test_fitter=fitter, test_covar=X)
