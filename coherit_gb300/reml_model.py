"""Model-level API: FitConfig and InfinitesimalREMLFitter (reml_model.py of GPU_REML).

Binds resident genotype streamers to ``fit_reml`` exactly as the reference
assembles its operator bundle for dense streamers (reml_model.py:962-1390):
one streamer (optionally partitioned into components, giving a one-pass
weighted H.V and a stacked K_g V), or several streamers (one per GRM), with
rare-variant sparse streamers appended after the dense ones as further GRMs
(reml_model.py:611-666, :1196-1290).  The
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
from .precond import (ProjectedCorePrecondConf, build_lowrank_basis, make_precond,
                      scalar_diag_from_precond_conf)
from .reml import REMLProbeCache, fit_reml
from .slq import default_workspace_bytes

logger = logging.getLogger(__name__)


@dataclasses.dataclass
class FitConfig:
    """The reference FitConfig (reml_model.py:34-83), same fields and defaults,
    plus the operator precisions of the GPU path.

    The admixture fields are accepted so that configs carry over, but an
    admixture-weighted fit raises NotImplementedError; ``cpu_threads``,
    ``ring_depth`` and ``source_build_chunk_width`` size the reference's host
    build threads and PCIe ring, which the resident operator does not have.
    """

    bed_prefix: str | Sequence[str] = ""
    sources: Sequence | None = None
    # Rare-variant sparse sources, one genetic component each
    # (reml_model.py:34-38, :611-666).
    rare_bed_prefix: str | Sequence[str] = ""
    rare_sources: Sequence | None = None
    vc_block_sizes: Sequence[int] | None = None
    component_variant_indices: Sequence[Sequence[int]] | None = None
    admix_weights: np.ndarray | None = None
    admix_component_names: Sequence[str] | None = None
    admix_residual_mode: str = "shared"
    # One (means, inv_sds) pair per dense source or BED prefix, or None.
    standardization_overrides: Sequence[tuple] | None = None
    sample_mask: np.ndarray | None = None
    call_width: int = 131072
    device: str | None = "auto"
    keep_host_stats: bool = True
    cpu_threads: int | None = None
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
    # Replicate fits with seeds seed + 9973 r; their mean and Monte-Carlo
    # standard errors are reported (reml_model.py:1891-1977).
    n_reml_reps: int = 1
    ring_depth: int | None = None
    source_build_chunk_width: int | None = None
    verbose: bool = True
    gpu_budget_bytes: float | None = None
    capture_reml_diagnostics: bool = False
    cache_reml_setup: bool = False
    strict_max_linesearch_trials: int = 3
    optimizer: str = "strict"
    precision: str = "bf16x3"
    sketch_precision: str = "bf16x1"
    # SLQ probe-batch workspace in bytes.  None: the reference's policy from
    # gpu_budget_bytes (256 MiB without one, at most 2 GiB), which batches 2
    # probes per operator application at n = 100,000 and 30 Lanczos steps.
    # A larger workspace batches more probes per application (each probe's
    # Lanczos recurrence is independent, so the results do not change) --
    # on a GPU whose HBM holds the whole probe block, fewer and wider
    # launches.
    slq_workspace_bytes: int | None = None
    # SMILE block-weighted GRMs (reml_model.py:42-53): exactly one W mode.
    smile_w_files: Sequence[str] | None = None
    smile_w_file_groups: Sequence[Sequence[str]] | None = None
    smile_weight_matrices: Sequence[np.ndarray] | None = None
    smile_weight_matrix_groups: Sequence[Sequence[np.ndarray]] | None = None
    smile_identity: bool = False
    smile_identity_block_size: int | None = None
    smile_normalization: str = "kernel_trace"
    smile_diag_mode: str = "mean"
    smile_strict_coverage: bool = True
    smile_w_device_cache_bytes: float | None = None
    smile_optimizer: str = "strict"
    smile_scoring_step_tol: float = 1e-4
    effect_pcg_tol: float = 1e-3


@dataclasses.dataclass
class FitResult:
    """Fields of the reference FitResult (reml_model.py:112-125) plus the wall time."""

    var_components: np.ndarray
    history: list
    rep_var_components: np.ndarray | None = None
    effects: "EffectEstimates | None" = None
    final_ai: np.ndarray | None = None
    final_grad: np.ndarray | None = None
    final_loglik: float | None = None
    diagnostics: dict | None = None
    heritability: float | None = None
    genetic_trace_atoms: np.ndarray | None = None
    residual_trace_atoms: np.ndarray | None = None
    monte_carlo_se_var: np.ndarray | None = None
    monte_carlo_se_h2: float | None = None
    elapsed_sec: float = 0.0


@dataclasses.dataclass
class EffectEstimates:
    """Post-REML effects on the standardised phenotype scale (reml_model.py:87-97)."""

    fixed_effects: torch.Tensor
    random_effect: torch.Tensor
    random_effect_components: tuple
    snp_effects: tuple
    pcg_rel_res: float
    pcg_iters: int
    y_mean: float
    y_scale: float


@dataclasses.dataclass
class PredictionEstimates:
    """Test-set predictions from effect estimates (reml_model.py:100-109)."""

    fixed_effect: torch.Tensor
    random_effect: torch.Tensor
    random_effect_components: tuple
    y_pred_std: torch.Tensor
    y_pred: torch.Tensor


def _validate_dense_prediction_streamers(train, test) -> None:
    """Train/test streamers must share the SNP set, call geometry, partition
    mode, cache-to-source SNP order and component layout (reml_model.py:223-272;
    the variant-metadata comparison against .bim/.pvar files is not made)."""
    if len(train) != len(test):
        raise ValueError(
            f"Prediction component count mismatch: expected {len(train)}, got {len(test)}.")
    for idx, (a, b) in enumerate(zip(train, test)):
        if int(a.m) != int(b.m):
            raise ValueError(f"Prediction SNP count mismatch for component {idx}: "
                             f"expected {int(a.m)}, got {int(b.m)}.")
        if int(a._n_calls) != int(b._n_calls):
            raise ValueError(f"Prediction call geometry mismatch for component {idx}: "
                             f"expected {int(a._n_calls)} calls, got {int(b._n_calls)}.")
        if not np.array_equal(np.asarray(a._call_snp_starts, np.int64),
                              np.asarray(b._call_snp_starts, np.int64)):
            raise ValueError(f"Prediction SNP call starts mismatch for component {idx}.")
        if not np.array_equal(np.asarray(a._call_true_widths, np.int32),
                              np.asarray(b._call_true_widths, np.int32)):
            raise ValueError(f"Prediction call widths mismatch for component {idx}.")
        partitioned = bool(getattr(a, "has_component_partition", False))
        if partitioned != bool(getattr(b, "has_component_partition", False)):
            raise ValueError(f"Prediction partitioning mode mismatch for component {idx}.")
        ca = getattr(a, "_cache_to_source_variant_indices", None)
        cb = getattr(b, "_cache_to_source_variant_indices", None)
        if ca is not None or cb is not None:
            if ca is None or cb is None:
                raise ValueError(f"Prediction variant-order mapping mismatch for component {idx}.")
            if not np.array_equal(np.asarray(ca, np.int64), np.asarray(cb, np.int64)):
                raise ValueError(f"Prediction source-variant order mismatch for component {idx}.")
        if partitioned and not np.array_equal(np.asarray(a._component_snp_offsets, np.int32),
                                              np.asarray(b._component_snp_offsets, np.int32)):
            raise ValueError("Prediction component block layout mismatch.")


def _solve_small_spd(A: torch.Tensor, b: torch.Tensor, *, base_jitter=1e-6, max_tries=8):
    """Host FP64 SPD solve with geometric jitter (reml_model.py:296-330)."""
    A_np = np.asarray(0.5 * (A + A.T).double().cpu().numpy())
    b_np = b.double().cpu().numpy().reshape(-1)
    p = A_np.shape[0]
    if p == 0:
        raise ValueError("solve_small_spd requires a non-empty square matrix.")
    scale = float(np.mean(np.abs(np.diag(A_np))))
    if not np.isfinite(scale) or scale <= 0.0:
        scale = 1.0
    for k in range(max_tries):
        try:
            L = np.linalg.cholesky(A_np + base_jitter * scale * (10.0 ** k) * np.eye(p))
        except np.linalg.LinAlgError:
            continue
        x = np.linalg.solve(L.T, np.linalg.solve(L, b_np))
        return torch.as_tensor(x, dtype=torch.float32, device=A.device)
    raise FloatingPointError("Failed to stabilize GLS normal equations with jitter escalation.")


def _prefix_list(prefix) -> list:
    items = list(prefix) if isinstance(prefix, (list, tuple)) else [prefix]
    return [str(p) for p in items if p]


@dataclasses.dataclass(frozen=True)
class _OperatorBundle:
    K_mvs: tuple
    diag_list: tuple
    weighted_hv: object
    stacked_kv: object
    projected_core_atoms: object | None = None


def _theta_ref_from_var_components(G: int, var_components_init=None) -> np.ndarray:
    """Weights of the preconditioner's reference kernel sum_g theta_ref,g K_g
    (reml_model.py:808-832): the first G variance components clamped at zero
    and normalised to sum 1; uniform 1/G without them or when they sum to
    zero or a non-finite value."""
    if var_components_init is None:
        th = np.ones(G, dtype=np.float32)
    else:
        th0 = np.asarray(var_components_init, dtype=np.float32).reshape(-1)
        if th0.size < G:
            raise ValueError(f"var_components_init length mismatch: expected at least {G}, "
                             f"got {th0.size}.")
        th = np.maximum(th0[:G], 0.0)
    total = float(np.sum(th))
    if total <= 0.0 or not np.isfinite(total):
        return np.full(G, 1.0 / max(1, G), dtype=np.float64)
    return (th / np.float32(total)).astype(np.float64)


class InfinitesimalREMLFitter:
    """Fit the infinitesimal (multi-)GRM REML model on resident genotypes."""

    def __init__(self, cfg: FitConfig, streamers: Sequence[GenoBlockStreamer] | None = None):
        self.cfg = cfg
        if cfg.admix_weights is not None:
            raise NotImplementedError(
                "Admixture-weighted GRMs are outside the GPU REML path; fit without admix_weights.")
        rare_prefixes = _prefix_list(cfg.rare_bed_prefix)
        has_rare = cfg.rare_sources is not None or bool(rare_prefixes)
        # One dense source split into components (reml_model.py:464-512).
        partitioned = cfg.vc_block_sizes is not None or cfg.component_variant_indices is not None
        if cfg.vc_block_sizes is not None and cfg.component_variant_indices is not None:
            raise ValueError("Use either vc_block_sizes or component_variant_indices, not both.")
        if partitioned and has_rare:
            raise ValueError("single-source component partitioning is currently supported only "
                             "for dense-only fits.")
        if streamers is None:
            smile = bool(cfg.smile_identity or cfg.smile_w_files or cfg.smile_w_file_groups
                         or cfg.smile_weight_matrices or cfg.smile_weight_matrix_groups)
            host_kw = dict(keep_host_stats=bool(cfg.keep_host_stats or smile),
                           build_threads=cfg.cpu_threads, ring_depth=cfg.ring_depth)
            dense_kw = dict(call_width=cfg.call_width, component_block_sizes=cfg.vc_block_sizes,
                            component_variant_indices=cfg.component_variant_indices,
                            sample_mask=cfg.sample_mask, device=cfg.device,
                            precision=cfg.precision,
                            source_build_chunk_width=cfg.source_build_chunk_width, **host_kw)
            overrides = (None if cfg.standardization_overrides is None
                         else list(cfg.standardization_overrides))
            # Sources take precedence over BED prefixes (reml_model.py:506-546).
            if cfg.sources is not None:
                items, what, one = list(cfg.sources), "dense sources", "dense source"
                make = lambda src, ov: GenoBlockStreamer(src, standardization_override=ov,
                                                         **dense_kw)
            else:
                items, what, one = _prefix_list(cfg.bed_prefix), "dense BED prefixes", "dense BED prefix"
                make = lambda p, ov: GenoBlockStreamer(bed_prefix=p, standardization_override=ov,
                                                       **dense_kw)
            if partitioned and len(items) != 1:
                raise ValueError(f"single-source component partitioning requires exactly one {one}.")
            if overrides is not None and len(overrides) != len(items):
                raise ValueError(f"standardization_overrides must match the number of {what}.")
            streamers = [make(item, None if overrides is None else overrides[i])
                         for i, item in enumerate(items)]
            if has_rare:
                from .sparse_stream import SparseGenoBlockStreamer

                rare_kw = dict(call_width=cfg.call_width, sample_mask=cfg.sample_mask,
                               device=cfg.device, gpu_budget_bytes=cfg.gpu_budget_bytes,
                               mixed_dense_sparse=bool(streamers), **host_kw)
                streamers += [SparseGenoBlockStreamer(src, **rare_kw)
                              for src in (cfg.rare_sources or ())]
                streamers += [SparseGenoBlockStreamer(bed_prefix=p, **rare_kw)
                              for p in rare_prefixes]
        self.streamers = list(streamers)
        if not self.streamers:
            raise ValueError("At least one dense or sparse genotype source is required.")
        sparse_flags = [bool(getattr(s, "has_sparse_backend", False)) for s in self.streamers]
        self._n_dense_streamers = sparse_flags.index(True) if any(sparse_flags) else len(sparse_flags)
        if any(not f for f in sparse_flags[self._n_dense_streamers:]):
            raise ValueError("Sparse (rare-variant) streamers must follow the dense streamers.")
        self._has_sparse = any(sparse_flags)
        self._sparse_streamers = tuple(self.streamers[self._n_dense_streamers:])
        ns = {int(s.n) for s in self.streamers}
        if len(ns) != 1:
            raise ValueError("all streamers must share the sample set")
        self.n = ns.pop()
        self.precond_conf: ProjectedCorePrecondConf | None = None
        # (scope, operator bundle) reused across fits when cache_reml_setup is
        # set, and the probe products that belong to that bundle.
        self._reml_fit_setup: tuple | None = None
        self._reml_probe_cache = REMLProbeCache()
        self._smile_operators = self._build_smile_operators()

    def _build_smile_operators(self) -> tuple:
        """SMILE W modes and their checks (reml_model.py:429-485)."""
        cfg = self.cfg
        present = {
            "identity": bool(cfg.smile_identity),
            "w_files": bool(cfg.smile_w_files),
            "w_file_groups": bool(cfg.smile_w_file_groups),
            "matrices": bool(cfg.smile_weight_matrices),
            "matrix_groups": bool(cfg.smile_weight_matrix_groups),
        }
        if present["w_files"] and present["matrices"]:
            raise ValueError("Use either smile_w_files or smile_weight_matrices, not both.")
        if sum(present.values()) > 1:
            raise ValueError(
                "Use only one SMILE W mode: identity, single W list, W file groups, "
                "single matrix list, or matrix groups.")
        if not any(present.values()):
            return ()
        if cfg.smile_normalization not in ("kernel_trace", "effective_rank"):
            raise ValueError("SMILE normalization must be 'kernel_trace' or 'effective_rank'.")
        if cfg.smile_diag_mode not in ("full", "mean"):
            raise ValueError("SMILE diag mode must be 'full' or 'mean'.")
        if cfg.vc_block_sizes is not None or cfg.component_variant_indices is not None:
            raise ValueError("SMILE block-W mode cannot be combined with component partitioning.")
        if self._has_sparse:
            raise ValueError("SMILE block-W mode is currently supported only for dense-only fits.")
        if len(self.streamers) != 1:
            raise ValueError("SMILE block-W mode requires exactly one dense genotype source.")
        from .smile_block_w import SmileBlockWeightedOperator, SmileMultiBlockWeightedOperator

        st = self.streamers[0]
        kw = dict(normalization=cfg.smile_normalization, strict_coverage=cfg.smile_strict_coverage,
                  diag_mode=cfg.smile_diag_mode)
        if present["identity"]:
            return (SmileBlockWeightedOperator.identity(
                st, block_size=cfg.smile_identity_block_size, **kw),)
        if present["matrices"]:
            return (SmileBlockWeightedOperator(st, list(cfg.smile_weight_matrices), **kw),)
        if present["w_files"]:
            return (SmileBlockWeightedOperator.from_weight_files(st, list(cfg.smile_w_files), **kw),)
        if present["matrix_groups"]:
            return SmileMultiBlockWeightedOperator.from_weight_matrix_groups(
                st, cfg.smile_weight_matrix_groups, **kw).operators
        return SmileMultiBlockWeightedOperator.from_weight_file_groups(
            st, cfg.smile_w_file_groups, **kw).operators

    # ------------------------------------------------------------ operators
    def _assemble_reml_operators(self) -> _OperatorBundle:
        prec = self.cfg.precision
        if self._smile_operators:
            # One X^T V pass shared by all SMILE GRMs (reml_model.py:1069-1164).
            from .smile_block_w import SmileMultiBlockWeightedOperator

            multi = SmileMultiBlockWeightedOperator(self._smile_operators)

            def atoms(U):
                KU = multi.stacked_kv(U)
                raw = torch.einsum("nr,gns->grs", U.to(KU.dtype), KU)
                return 0.5 * (raw + raw.transpose(-1, -2))

            return _OperatorBundle(
                K_mvs=tuple((lambda V, op=op: op.kv(V)) for op in self._smile_operators),
                diag_list=tuple(op.diag() for op in self._smile_operators),
                weighted_hv=multi.weighted_hv, stacked_kv=multi.stacked_kv,
                projected_core_atoms=atoms)
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

    def _make_effect_precond(self, ops: _OperatorBundle, theta_g, theta_e):
        """M^{-1} at the given variance components (reml_model.py:1443-1457)."""
        if self.precond_conf is None:
            return None
        dev = self.streamers[0].dev
        tg = torch.as_tensor(np.asarray(theta_g, float).reshape(-1), dtype=torch.float32, device=dev)
        te = torch.as_tensor(np.asarray(theta_e, float).reshape(-1), dtype=torch.float32, device=dev)
        diag_H = scalar_diag_from_precond_conf(self.precond_conf, tg, te)
        if diag_H is None:
            stack = torch.stack([torch.as_tensor(d, dtype=torch.float32, device=dev).expand(self.n)
                                 for d in ops.diag_list])
            diag_H = te[0] + torch.tensordot(tg, stack, dims=1)
        return make_precond(self.precond_conf, tg, diag_H, eps=self.cfg.pcg_ridge)

    def _ensure_projected_core_precond_ready(self, ops: _OperatorBundle, var_components_init=None):
        if self.precond_conf is None and self.cfg.precond_rank > 0:
            self._build_projected_core_precond(ops, var_components_init)

    def _build_projected_core_precond(self, ops: _OperatorBundle, var_components_init=None,
                                      theta_ref=None) -> ProjectedCorePrecondConf:
        """Nystrom basis of the reference kernel + projected cores (reml_model.py:863-960)."""
        cfg = self.cfg
        G = len(ops.K_mvs)
        atoms = np.asarray([float(torch.as_tensor(d).double().mean()) for d in ops.diag_list])
        if theta_ref is None:
            theta_ref = _theta_ref_from_var_components(G, var_components_init)
        sk = cfg.sketch_precision
        if self._smile_operators:
            def K_ref(V):
                return ops.weighted_hv(theta_ref, None, V)
        elif len(self.streamers) == 1 and not self._has_sparse:
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
    def _setup_scope(self) -> tuple:
        """Objects a cached operator bundle and its probe products depend on
        (reml_model.py:1849-1871): the SMILE operators, every streamer and its
        statistics arrays.  Streamers replace these arrays when their
        standardisation changes, so an identity comparison detects it."""
        items = list(self._smile_operators)
        for st in self.streamers:
            items.append(st)
            items.extend(getattr(st, name, None) for name in (
                "_means_by_call", "_inv_by_call", "_component_snp_offsets",
                "_component_eff_m_host", "_eff_m_const", "_cache_to_source_variant_indices"))
        return tuple(items)

    def close(self) -> None:
        """Drop the cached set-up and close every streamer (reml_model.py:1818-1838)."""
        self._reml_fit_setup = None
        self._reml_probe_cache = REMLProbeCache()
        self.precond_conf = None
        for st in getattr(self, "streamers", ()):
            close_streamer = getattr(st, "close", None)
            if not callable(close_streamer):
                continue
            try:
                close_streamer()
            except (OSError, RuntimeError, ValueError, BufferError):
                logger.debug("Failed to close fitter streamer.", exc_info=True)
        self.streamers = []
        self._has_sparse = False
        self._sparse_streamers = ()
        self._smile_operators = ()

    def fit_infinitesimal(self, y, covar=None, h2_init: float = 0.5, var_components_init=None,
                          estimate_effects: bool = False, mean_information=None,
                          *, slq_probes=None, trace_probes=None, precond: bool = True):
        """AI-REML fit of the variance components (reml_model.py:1840-2010).

        With ``n_reml_reps`` > 1 the fit is repeated with seeds
        ``seed + 9973 r`` and the mean is returned with Monte-Carlo standard
        errors of the components and of h2.  ``estimate_effects`` adds the
        BLUP and SNP effects at the fitted components.  ``slq_probes`` /
        ``trace_probes`` fix the probe matrices (then replicates only differ
        through their seeds' unused streams).
        """
        t0 = time.time()
        cfg = self.cfg
        if not self.streamers:
            raise RuntimeError("InfinitesimalREMLFitter is closed.")
        if mean_information is not None:
            raise NotImplementedError("sparse mean information is outside the GPU REML path")
        if cfg.cache_reml_setup:
            scope = self._setup_scope()
            setup = self._reml_fit_setup
            if setup is None or len(setup[0]) != len(scope) or any(
                    old is not new for old, new in zip(setup[0], scope)):
                self._reml_fit_setup = (scope, self._assemble_reml_operators())
                self._reml_probe_cache = REMLProbeCache()
            ops = self._reml_fit_setup[1]
        else:
            ops = self._assemble_reml_operators()
        G = len(ops.K_mvs)
        if precond:
            # Built once per fitter, at the first fit (reml_model.py:1392-1407);
            # multi-GRM fits refresh it as theta moves.
            self._ensure_projected_core_precond_ready(ops, var_components_init)
        conf = self.precond_conf if precond and cfg.precond_rank > 0 else None
        refresh = None
        if conf is not None and G > 1:
            refresh = lambda p: self._build_projected_core_precond(ops, var_components_init=p)
        reps = []
        n_reps = max(1, int(cfg.n_reml_reps))
        for r in range(n_reps):
            reps.append(fit_reml(
                y=y, K_mvs=ops.K_mvs, diag_list=ops.diag_list, covar=covar,
                n_rand_vec=cfg.n_rand_vec, maxiter=cfg.max_pcg_iters, seed=cfg.seed + r * 9973,
                h2_init=h2_init, param_init=var_components_init, minq_iter=cfg.minq_iter,
                slq_samples=cfg.slq_samples, slq_m=cfg.slq_m, slq_mode=cfg.slq_mode,
                slq_workspace_bytes=(int(cfg.slq_workspace_bytes) if cfg.slq_workspace_bytes
                                     else default_workspace_bytes(cfg.gpu_budget_bytes)),
                precond_conf=conf, slq_precond_conf=conf, precond_refresh_fn=refresh,
                precond_eps=cfg.pcg_ridge, weighted_hv=ops.weighted_hv, stacked_kv=ops.stacked_kv,
                optimizer=cfg.smile_optimizer if self._smile_operators else cfg.optimizer,
                scoring_step_tol=(cfg.smile_scoring_step_tol if self._smile_operators else 1e-4),
                pcg_tol=cfg.reml_pcg_tol,
                response_is_standardized=cfg.response_is_standardized,
                unit_variance_components=cfg.unit_variance_components,
                max_linesearch_trials=cfg.strict_max_linesearch_trials, return_diagnostics=True,
                verbose=cfg.verbose,
                probe_cache=self._reml_probe_cache if cfg.cache_reml_setup else None,
                device=self.streamers[0].dev,
                slq_probes=slq_probes, trace_probes=trace_probes,
            ))
        param, history, diag = reps[0]
        # Unit-variance components report no trace atoms (reml_model.py:1876-1889).
        ga, ra = (None if diag.get(k) is None else np.asarray(diag[k], np.float64)
                  for k in ("genetic_trace_atoms", "residual_trace_atoms"))

        def reported_h2(theta):
            theta = np.asarray(theta, np.float64)
            if cfg.unit_variance_components:
                gen, res = np.sum(theta[..., :G], axis=-1), np.sum(theta[..., G:], axis=-1)
            else:
                gen, res = theta[..., :G] @ ga, theta[..., G:] @ ra
            return gen / np.maximum(gen + res, 1e-8)

        rep_vc = se_var = se_h2 = None
        if n_reps > 1:
            rep_vc = np.stack([np.asarray(p, np.float64) for p, _, _ in reps])
            param = rep_vc.mean(axis=0)
            denom = float(n_reps * (n_reps - 1))
            se_var = np.sqrt(np.maximum(0.0, np.sum((rep_vc - param) ** 2, axis=0) / denom))
            h2_reps = reported_h2(rep_vc)
            se_h2 = float(np.sqrt(max(0.0, float(np.sum((h2_reps - h2_reps.mean()) ** 2)) / denom)))
            # The AI, gradient and likelihood of one replicate do not describe the mean.
            diag = None
        h2 = float(reported_h2(param))
        effects = (self.estimate_effects(y, var_components=param, covar=covar)
                   if estimate_effects else None)
        return FitResult(
            var_components=param, history=history, rep_var_components=rep_vc, effects=effects,
            final_ai=None if diag is None else np.asarray(diag["ai"]),
            final_grad=None if diag is None else np.asarray(diag["grad"]),
            final_loglik=None if diag is None else float(diag["loglik"]),
            diagnostics=diag if cfg.capture_reml_diagnostics else None,
            heritability=h2, genetic_trace_atoms=ga, residual_trace_atoms=ra,
            monte_carlo_se_var=se_var, monte_carlo_se_h2=se_h2, elapsed_sec=time.time() - t0)


    # ------------------------------------------------------------ effects
    def _estimate_snp_effects(self, alpha: torch.Tensor, theta_g) -> tuple:
        """Per-component SNP effects beta_g with Z_g beta_g = theta_g K_g alpha
        (reml_model.py:1459-1540): theta_g/m_eff,g Z_g^T alpha."""
        tg = np.asarray(theta_g, float).reshape(-1)
        if self._smile_operators:
            if tg.size != len(self._smile_operators):
                raise ValueError(
                    f"theta_g must have length {len(self._smile_operators)} for SMILE effects.")
            return tuple(op.snp_effects(alpha, tg[i]) for i, op in enumerate(self._smile_operators))
        if len(self.streamers) == 1 and self.streamers[0].n_components > 1:
            st = self.streamers[0]
            xt = st.xtv(alpha, normalize=False)
            out = []
            for g in range(st.n_components):
                a, b = int(st._component_snp_offsets[g]), int(st._component_snp_offsets[g + 1])
                eff = float(st._component_eff_m_host[g])
                out.append(xt[a:b] * (tg[g] / eff) if eff > 0 else torch.zeros_like(xt[a:b]))
            return tuple(out)
        return tuple(float(tg[g]) * st.xtv(alpha, normalize=True)
                     for g, st in enumerate(self.streamers))

    def estimate_effects(self, y, *, var_components, covar=None) -> EffectEstimates:
        """Fixed effects, BLUP random effect and SNP effects at the given
        variance components (reml_model.py:1543-1644)."""
        if not self.streamers:
            raise RuntimeError("estimate_effects requires initialized streamers.")
        from .pcg import pcg_solve
        from .reml import standardize_response

        ops = self._assemble_reml_operators()
        G = len(ops.K_mvs)
        theta = np.asarray(var_components, dtype=np.float64).reshape(-1)
        if theta.size != G + 1:
            raise ValueError(f"var_components length mismatch: expected {G + 1}, got {theta.size}.")
        theta_g, theta_e = theta[:-1], theta[-1]
        self._ensure_projected_core_precond_ready(ops, var_components_init=theta)
        dev = self.streamers[0].dev
        y_t = torch.as_tensor(y, dtype=torch.float32).reshape(-1).to(dev)
        if self.cfg.response_is_standardized:
            if not bool(torch.all(torch.isfinite(y_t))):
                raise ValueError("Phenotype contains non-finite values.")
            y_std, y_mean, y_scale = y_t, 0.0, 1.0
        else:
            y_std, y_mean, y_scale = standardize_response(y_t)
        xmat = None
        if covar is not None:
            xmat = torch.as_tensor(covar, dtype=torch.float32).to(dev)
            if xmat.ndim == 1:
                xmat = xmat[:, None]
            if xmat.numel() == 0:
                xmat = None
        Hv = self._make_hv(ops, theta_g, theta_e)
        M = self._make_effect_precond(ops, theta_g, theta_e)
        rhs = y_std[:, None] if xmat is None else torch.cat([y_std[:, None], xmat], dim=1)
        rhs = rhs.contiguous()
        X0 = M(rhs) if M is not None else torch.zeros_like(rhs)
        tol = float(self.cfg.effect_pcg_tol)
        sol, rel, iters = pcg_solve(Hv, rhs, M=M, tol=tol, maxiter=self.cfg.max_pcg_iters, X0=X0)
        if not bool(torch.all(torch.isfinite(sol))):
            raise FloatingPointError("Non-finite PCG solution encountered in estimate_effects.")
        rel_host = float(torch.as_tensor(rel).double().max())
        if not np.isfinite(rel_host) or rel_host > tol * 1.05:
            raise FloatingPointError(
                f"Effect-estimation PCG did not converge: relative residual={rel_host:.3e}, "
                f"tolerance={tol:.3e}, iterations={int(iters)}/{int(self.cfg.max_pcg_iters)}.")
        Hinv_y = sol[:, 0]
        if xmat is not None:
            Hinv_x = sol[:, 1:]
            fixed = _solve_small_spd(xmat.T @ Hinv_x, xmat.T @ Hinv_y)
            alpha = Hinv_y - Hinv_x @ fixed
        else:
            fixed = torch.empty(0, dtype=torch.float32, device=dev)
            alpha = Hinv_y
        alpha = alpha.contiguous()
        if ops.stacked_kv is not None:
            Ka = ops.stacked_kv(alpha[:, None])[..., 0]
        else:
            Ka = torch.stack([mv(alpha) for mv in ops.K_mvs], dim=0)
        tg_t = torch.as_tensor(theta_g, dtype=torch.float32, device=dev)
        comps = tuple(float(theta_g[g]) * Ka[g] for g in range(G))
        return EffectEstimates(
            fixed_effects=fixed, random_effect=torch.sum(tg_t[:, None] * Ka, dim=0),
            random_effect_components=comps, snp_effects=self._estimate_snp_effects(alpha, theta_g),
            pcg_rel_res=rel_host, pcg_iters=int(iters), y_mean=float(y_mean),
            y_scale=float(y_scale))

    def predict(self, effects: EffectEstimates, *, test_fitter: "InfinitesimalREMLFitter",
                test_covar=None) -> PredictionEstimates:
        """X_test b + Z_test beta on the test samples with the training
        standardisation (reml_model.py:1646-1818): one Z b pass per test
        streamer, the components as columns of b."""
        if self._has_sparse or getattr(test_fitter, "_has_sparse", False):
            raise NotImplementedError(
                "Prediction currently supports dense genotype paths only; sparse test prediction "
                "is not implemented.")
        if not self.streamers or not test_fitter.streamers:
            raise RuntimeError("Prediction requires initialized training and test streamers.")
        _validate_dense_prediction_streamers(self.streamers, test_fitter.streamers)
        if len(self.streamers) == 1 and self.streamers[0].n_components > 1:
            expected = self.streamers[0].n_components
        elif self._smile_operators:
            expected = len(self._smile_operators)
        else:
            expected = len(self.streamers)
        if len(effects.snp_effects) != expected:
            raise ValueError("Prediction SNP-effect component count mismatch: "
                             f"expected {expected}, got {len(effects.snp_effects)}.")
        for a, b in zip(self.streamers, test_fitter.streamers):
            b.set_standardization(a._means_host, a._inv_sds_host)
        st_test0 = test_fitter.streamers[0]
        dev = st_test0.dev
        n_test = int(st_test0.n)
        beta = torch.as_tensor(effects.fixed_effects, dtype=torch.float32).reshape(-1).to(dev)
        X_test = None
        if test_covar is not None:
            X_test = torch.as_tensor(test_covar, dtype=torch.float32).to(dev)
            if X_test.ndim == 1:
                X_test = X_test[:, None]
            if X_test.ndim != 2 or X_test.shape[0] != n_test:
                raise ValueError("Prediction covariates must be a 2D matrix with one row per test sample.")
            if not bool(torch.all(torch.isfinite(X_test))):
                raise ValueError("Prediction covariates contain non-finite values.")
        if beta.numel() > 0:
            if X_test is None:
                raise ValueError("Prediction requires test covariates aligned to the training design matrix.")
            if X_test.shape[1] != beta.numel():
                raise ValueError(f"Prediction covariate width mismatch: expected {beta.numel()}, "
                                 f"got {X_test.shape[1]}.")
            fixed_effect = X_test @ beta
        else:
            fixed_effect = torch.zeros(n_test, dtype=torch.float32, device=dev)
        if len(self.streamers) == 1:
            st_tr = self.streamers[0]
            B = torch.zeros((int(st_tr.m), expected), dtype=torch.float32, device=dev)
            if st_tr.n_components > 1 and not self._smile_operators:
                for g in range(expected):
                    a, b = int(st_tr._component_snp_offsets[g]), int(st_tr._component_snp_offsets[g + 1])
                    B[a:b, g] = torch.as_tensor(effects.snp_effects[g], dtype=torch.float32).to(dev).reshape(-1)
            else:
                for g in range(expected):
                    bg = torch.as_tensor(effects.snp_effects[g], dtype=torch.float32).to(dev).reshape(-1)
                    if bg.numel() != int(st_tr.m):
                        raise ValueError(f"SNP-effect length mismatch: expected {int(st_tr.m)}, "
                                         f"got {bg.numel()}.")
                    B[:, g] = bg
            comp = st_test0.zxb(B)
            components = tuple(comp[:, g] for g in range(expected))
        else:
            components = tuple(
                st.zxb(torch.as_tensor(b, dtype=torch.float32).to(dev).reshape(-1))
                for st, b in zip(test_fitter.streamers, effects.snp_effects))
        random_effect = torch.stack(components, dim=0).sum(0)
        y_pred_std = fixed_effect + random_effect
        return PredictionEstimates(
            fixed_effect=fixed_effect, random_effect=random_effect,
            random_effect_components=components, y_pred_std=y_pred_std,
            y_pred=float(effects.y_mean) + float(effects.y_scale) * y_pred_std)


__all__ = ["FitConfig", "FitResult", "InfinitesimalREMLFitter", "EffectEstimates",
           "PredictionEstimates"]
