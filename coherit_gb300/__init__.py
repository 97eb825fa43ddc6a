"""coherit_gb300 -- GB300-native (sm_103a) matrix-free REML hot path.

A drop-in for GPU_REML's genotype operator and the solvers built on it:
``kv_impl``, ``geno_stream``, ``block_backend``, ``pcg``, ``precond``,
``slq`` and ``reml`` keep the reference's module names and call surface,
with 2-bit genotypes resident in HBM and the operator running as
hand-written CUDA (tcgen05 tensor cores) behind the C ABI of
``include/coherit_gpu.h``.  Names are exported lazily like the reference
package (__init__.py:6-48).
"""
from __future__ import annotations

import importlib

_EXPORTS: dict[str, str] = {
    "GenoBlockStreamer": ".geno_stream",
    "BedBlockStreamer": ".geno_stream",
    "ArraySource": ".geno_stream",
    "SyntheticSource": ".geno_stream",
    "BedSource": ".bed",
    "DensePackedBlockDescriptor": ".block_backend",
    "Sparse12BlockDescriptor": ".block_backend",
    "ProjectedCorePrecondConf": ".precond",
    "ProjectedCoreRuntime": ".precond",
    "build_lowrank_basis": ".precond",
    "build_projected_core_runtime": ".precond",
    "make_precond": ".precond",
    "make_projected_core_precond": ".precond",
    "projected_core_apply_invsqrt": ".precond",
    "projected_core_logdet": ".precond",
    "InfinitesimalREMLFitter": ".reml_model",
    "FitConfig": ".reml_model",
    "FitResult": ".reml_model",
    "EffectEstimates": ".reml_model",
    "PredictionEstimates": ".reml_model",
    "pcg_solve": ".pcg",
    "fit_reml": ".reml",
    "standardize_response": ".reml",
    "REMLServer": ".serving",
    "SmileBlockWeight": ".smile_block_w",
    "SmileBlockWeightedOperator": ".smile_block_w",
    "SmileMultiBlockWeightedOperator": ".smile_block_w",
    "load_rds_matrix": ".smile_block_w",
    "load_weight_matrix": ".smile_block_w",
    "validate_weight_matrix": ".smile_block_w",
    "ServeResult": ".serving",
    "GWASSummary": ".gwas",
    "run_continuous_gwas": ".gwas",
    "marginal_scan": ".gwas",
    "solve_hinv_columns_batched": ".hinv",
    "compute_projected_hinv_vector": ".hinv",
    "SparseGenoBlockStreamer": ".sparse_stream",
    "SyntheticRareSource": ".sparse_stream",
}

__all__ = list(_EXPORTS)


def __getattr__(name: str):
    module_name = _EXPORTS.get(name)
    if module_name is None:
        raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
    module = importlib.import_module(module_name, __name__)
    value = getattr(module, name)
    globals()[name] = value
    return value
