"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol."""
import ctypes
import re
from pathlib import Path

from coherit_gb300 import _lib, build_ext

HEADER = Path(__file__).resolve().parents[1] / "include" / "coherit_gpu.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(coherit_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_loads():
    path = build_ext.build()
    assert path.exists()
    lib = ctypes.CDLL(str(path))
    assert lib.coherit_version() == 1


def test_every_declared_symbol_is_exported_and_bound():
    lib = _lib.load()
    declared = declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in coherit_gpu.h but not exported"
    assert set(declared) == set(_lib.exported_symbols())


def test_status_mapping():
    import pytest

    with pytest.raises(ValueError):
        _lib.check(_lib.E_SHAPE)
    with pytest.raises(IndexError):
        _lib.check(_lib.E_INDEX)
    with pytest.raises(FloatingPointError):
        _lib.check(_lib.E_NONFINITE)
    with pytest.raises(RuntimeError):
        _lib.check(_lib.E_CLOSED)
    with pytest.raises(FloatingPointError):
        _lib.check(_lib.E_NOT_CONVERGED)
    with pytest.raises(MemoryError):
        _lib.check(_lib.E_OOM)
    for code in (_lib.E_TIMEOUT, _lib.E_CUDA, _lib.E_UNSUPPORTED):
        with pytest.raises(RuntimeError, match=f"status {code}"):
            _lib.check(code, "op")
    _lib.check(_lib.OK)


def test_package_exports_resolve():
    import coherit_gb300

    for name in coherit_gb300.__all__:
        assert getattr(coherit_gb300, name) is not None, name
    # The reference package's exports (__init__.py:6-48) that belong to the
    # operator, solver, model, SMILE and GWAS layers.
    hot_path = {
        "GenoBlockStreamer", "BedBlockStreamer", "SparseGenoBlockStreamer",
        "DensePackedBlockDescriptor", "Sparse12BlockDescriptor", "ProjectedCorePrecondConf",
        "ProjectedCoreRuntime", "build_lowrank_basis", "build_projected_core_runtime",
        "make_precond", "make_projected_core_precond", "projected_core_apply_invsqrt",
        "projected_core_logdet", "InfinitesimalREMLFitter", "FitConfig", "FitResult",
        "EffectEstimates", "PredictionEstimates", "pcg_solve", "fit_reml",
        "compute_projected_hinv_vector", "GWASSummary", "run_continuous_gwas",
        "SmileBlockWeight", "SmileBlockWeightedOperator", "load_rds_matrix",
        "load_weight_matrix", "validate_weight_matrix",
    }
    assert hot_path <= set(coherit_gb300.__all__)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built library every entry point refuses."""
    import pytest

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(build_ext, "LIB_PATH", tmp_path / "libcoherit_gpu.so")
    with pytest.raises(RuntimeError, match="CUDA library not found"):
        _lib.load(build_if_missing=False)


def test_null_handle_is_rejected_without_gpu():
    lib = _lib.load()
    assert lib.coherit_geno_info(None, None, None, None, None, None, None, None) == _lib.E_CLOSED
    assert lib.coherit_geno_check(None, None) == _lib.E_CLOSED
