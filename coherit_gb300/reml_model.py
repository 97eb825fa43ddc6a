"""Model-level API: FitConfig and InfinitesimalREMLFitter (reml_model.py of GPU_REML).

Binds resident genotype streamers to ``fit_reml`` exactly as the reference
assembles its operator bundle for dense streamers (reml_model.py:962-1390):
one streamer (optionally partitioned into components, giving a one-pass
weighted H.V and a stacked K_g V), or several streamers (one per GRM).  The
projected-core preconditioner is built from a Nystrom basis of the
reference kernel sum_g theta_ref,g K_g and the per-component projected cores
(reml_model.py:863-960).
"""
from __future__ import annotations

import dataclasses
import logging
import time
from typing import Optional, Sequence

import numpy as np
import torch

from .geno_stream import GenoBlockStreamer
from .precond import ProjectedCorePrecondConf, build_lowrank_basis
from .reml import REMLProbeCache, fit_reml
from .slq import default_workspace_bytes

logger = logging.getLogger(__name__)


@dataclasses.dataclass
class FitConfig:
    """Subset of the reference FitConfig (reml_model.py:34-83) used by the GPU path."""

    sources: Sequence | None = None
    vc_block_sizes: Sequence[int] | None = None
    component_variant_indices: Sequence[Sequence[int]] | None = None
    sample_mask: np.ndarray | None = None
    call_width: int = 131072
    device: str | None = "auto"
    n_rand_vec: int = 100
    max_pcg_iters: int = 400
    minq_iter: int = 50
    seed: int = 0
    slq_samples: int = 4
    slq_m: int = 8
    slq_mode: str = "projected_core_residual"
    precond_rank: int = 500
    pcg_ridge: float = 1e-6
    reml_pcg_tol: float = 1e-3
    response_is_standardized: bool = False
    unit_variance_components: bool = False
    verbose: bool = False
    gpu_budget_bytes: float | None = None
    capture_reml_diagnostics: bool = False
    cache_reml_setup: bool = False
    strict_max_linesearch_trials: int = 3
    optimizer: str = "strict"
    precision: str = "bf16x3"
    sketch_precision: str = "bf16x1"


@dataclasses.dataclass
class FitResult:
    var_components: np.ndarray
    history: list
    heritability: float | None = None
    genetic_trace_atoms: np.ndarray | None = None
    residual_trace_atoms: np.ndarray | None = None
    diagnostics: dict | None = None
    final_loglik: float | None = None
    elapsed_sec: float = 0.0


@dataclasses.dataclass(frozen=True)
class _OperatorBundle:
    K_mvs: tuple
    diag_list: tuple
    weighted_hv: object
    stacked_kv: object
    projected_core_atoms: object | None = None


class InfinitesimalREMLFitter:
    """Fit the infinitesimal (multi-)GRM REML model on resident genotypes."""

    def __init__(self, cfg: FitConfig, streamers: Sequence[GenoBlockStreamer] | None = None):
        self.cfg = cfg
        if streamers is None:
            if not cfg.sources:
                raise ValueError("FitConfig.sources or explicit streamers are required.")
            streamers = [
                GenoBlockStreamer(
                    src, call_width=cfg.call_width, component_block_sizes=cfg.vc_block_sizes,
                    component_variant_indices=cfg.component_variant_indices,
                    sample_mask=cfg.sample_mask, device=cfg.device, precision=cfg.precision)
                for src in cfg.sources
            ]
        self.streamers = list(streamers)
        if not self.streamers:
            raise ValueError("at least one streamer is required")
        ns = {int(s.n) for s in self.streamers}
        if len(ns) != 1:
            raise ValueError("all streamers must share the sample set")
        self.n = ns.pop()
        self.precond_conf: ProjectedCorePrecondConf | None = None
        self._probe_cache = REMLProbeCache() if cfg.cache_reml_setup else None
        self._ops: _OperatorBundle | None = None

    # ------------------------------------------------------------ operators
    def _assemble_reml_operators(self) -> _OperatorBundle:
        prec = self.cfg.precision
        if len(self.streamers) == 1 and self.streamers[0].n_components > 1:
            st = self.streamers[0]
            G = st.n_components
            K_mvs = tuple(
                (lambda V, g=g: st.component_kv(V, g, precision=prec)) for g in range(G))
            return _OperatorBundle(
                K_mvs=K_mvs,
                diag_list=tuple(st.component_diag_list()),
                weighted_hv=lambda tg, te, V: st.weighted_component_hv(tg, te, V, precision=prec),
                stacked_kv=lambda V: st.stacked_component_kv(V, precision=prec),
                projected_core_atoms=lambda U: st.build_projected_core_atoms(U, subtract_identity=False),
            )
        sts = self.streamers
        K_mvs = tuple((lambda V, s=s: s.kv(V, precision=prec)) for s in sts)
        diag_list = tuple(s.diag() for s in sts)
        if len(sts) == 1:
            st = sts[0]

            def whv(tg, te, V):
                return st.weighted_component_hv(tg, te, V, precision=prec)

            return _OperatorBundle(K_mvs, diag_list, whv, None)

        def whv_multi(tg, te, V):
            acc = None
            for g, s in enumerate(sts):
                term = s.weighted_component_hv([float(tg[g])], float(te) if (g == 0 and te is not None) else None,
                                               V, precision=prec)
                acc = term if acc is None else acc + term
            return acc

        return _OperatorBundle(K_mvs, diag_list, whv_multi,
                               lambda V: torch.stack([s.kv(V, precision=prec) for s in sts]))

    def _make_hv(self, ops: _OperatorBundle, theta_g, theta_e):
        """H.V closure for downstream solves (reml_model.py:1431-1441)."""
        tg = np.asarray(theta_g, float).reshape(-1)
        te = float(np.asarray(theta_e, float).reshape(-1)[0])
        if ops.weighted_hv is not None:
            return lambda V: ops.weighted_hv(tg, te, V)
        return lambda V: sum(float(tg[i]) * mv(V) for i, mv in enumerate(ops.K_mvs)) + te * V

    def _build_projected_core_precond(self, ops: _OperatorBundle, var_components_init=None,
                                      theta_ref=None) -> ProjectedCorePrecondConf:
        """Nystrom basis of the reference kernel + projected cores (reml_model.py:863-960)."""
        cfg = self.cfg
        G = len(ops.K_mvs)
        atoms = np.asarray([float(d) for d in ops.diag_list])
        if theta_ref is None:
            if var_components_init is not None:
                theta_ref = np.asarray(var_components_init, float)[:G]
            else:
                theta_ref = np.where(atoms > 0, 1.0 / max(float(np.sum(atoms)), 1e-12), 0.0)
        theta_ref = np.asarray(theta_ref, float)
        sk = cfg.sketch_precision
        if len(self.streamers) == 1:
            st = self.streamers[0]
            eff = st._component_eff_m_host.astype(np.float64)

            def K_ref(V):
                scale = np.where(eff > 0, theta_ref / np.where(eff > 0, eff, 1), 0.0)
                return st._kv_raw(V, comp_scale=scale, precision=sk)
        else:
            def K_ref(V):
                acc = None
                for g, s in enumerate(self.streamers):
                    t = float(theta_ref[g]) * s.kv(V, precision=sk)
                    acc = t if acc is None else acc + t
                return acc
        dev = self.streamers[0].dev
        rank = int(min(cfg.precond_rank, self.n, sum(s.m for s in self.streamers)))
        U, evals = build_lowrank_basis(K_ref, self.n, rank, key=cfg.seed + 4321, device=dev)
        r = int(U.shape[1])
        eye = torch.eye(r, dtype=U.dtype, device=dev)
        if G == 1:
            raw = torch.diag(evals.to(U.dtype))[None]
        elif ops.projected_core_atoms is not None:
            raw = ops.projected_core_atoms(U)
        else:
            KU = ops.stacked_kv(U)
            raw = torch.einsum("nr,gns->grs", U, KU)
        core = 0.5 * (raw + raw.transpose(-1, -2))
        core = core - torch.as_tensor(atoms, dtype=U.dtype, device=dev)[:, None, None] * eye[None]
        conf = ProjectedCorePrecondConf(
            U=U, core_atoms=core, total_rank=r, n_grm=G, diag_mode="scalar_identity",
            diag_atoms=torch.as_tensor(atoms, dtype=torch.float32, device=dev),
            residual_diag_atoms=torch.ones(1, dtype=torch.float32, device=dev), identity=eye)
        self.precond_conf = conf
        return conf

    # ------------------------------------------------------------------ fit
    def fit_infinitesimal(self, y, covar=None, h2_init: float = 0.5, var_components_init=None,
                          *, slq_probes=None, trace_probes=None, precond: bool = True):
        t0 = time.time()
        cfg = self.cfg
        if self._ops is None or not cfg.cache_reml_setup:
            self._ops = self._assemble_reml_operators()
        ops = self._ops
        G = len(ops.K_mvs)
        if precond and cfg.precond_rank > 0 and (self.precond_conf is None or not cfg.cache_reml_setup):
            self._build_projected_core_precond(ops, var_components_init)
        conf = self.precond_conf if precond and cfg.precond_rank > 0 else None
        refresh = None
        if conf is not None and G > 1:
            refresh = lambda p: self._build_projected_core_precond(ops, theta_ref=np.asarray(p)[:G])
        out = fit_reml(
            y=y, K_mvs=ops.K_mvs, diag_list=ops.diag_list, covar=covar,
            n_rand_vec=cfg.n_rand_vec, maxiter=cfg.max_pcg_iters, seed=cfg.seed, h2_init=h2_init,
            param_init=var_components_init, minq_iter=cfg.minq_iter, slq_samples=cfg.slq_samples,
            slq_m=cfg.slq_m, slq_mode=cfg.slq_mode,
            slq_workspace_bytes=default_workspace_bytes(cfg.gpu_budget_bytes),
            precond_conf=conf, slq_precond_conf=conf, precond_refresh_fn=refresh,
            precond_eps=cfg.pcg_ridge, weighted_hv=ops.weighted_hv, stacked_kv=ops.stacked_kv,
            optimizer=cfg.optimizer, pcg_tol=cfg.reml_pcg_tol,
            response_is_standardized=cfg.response_is_standardized,
            unit_variance_components=cfg.unit_variance_components,
            max_linesearch_trials=cfg.strict_max_linesearch_trials, return_diagnostics=True,
            verbose=cfg.verbose, probe_cache=self._probe_cache, device=self.streamers[0].dev,
            slq_probes=slq_probes, trace_probes=trace_probes,
        )
        param, history, diag = out
        ga = diag.get("genetic_trace_atoms")
        ra = diag.get("residual_trace_atoms")
        if cfg.unit_variance_components:
            gen, res = float(np.sum(param[:G])), float(np.sum(param[G:]))
        else:
            gen, res = float(param[:G] @ ga), float(param[G:] @ ra)
        h2 = gen / max(gen + res, 1e-8)
        return FitResult(var_components=param, history=history, heritability=h2,
                         genetic_trace_atoms=ga, residual_trace_atoms=ra,
                         diagnostics=diag if cfg.capture_reml_diagnostics else None,
                         final_loglik=float(diag["loglik"]), elapsed_sec=time.time() - t0)


__all__ = ["FitConfig", "FitResult", "InfinitesimalREMLFitter"]
