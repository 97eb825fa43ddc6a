"""ctypes binding of ``libcoherit_gpu.so`` and status -> exception mapping.

The library is built in-tree (``coherit_gb300/libcoherit_gpu.so``) by
``coherit_gb300.build_ext``.  Every call goes through :func:`check`, which
turns the C status codes into the exception types the reference raises for
the same conditions (ValueError for shapes, IndexError for component ids,
FloatingPointError for numerical failure, RuntimeError for a closed handle).
There is no CPU fallback: importing the operator without the library raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build_ext

OK = 0
E_SHAPE = 1
E_NONFINITE = 2
E_NOT_CONVERGED = 3
E_OOM = 4
E_TIMEOUT = 5
E_CLOSED = 6
E_CUDA = 7
E_INDEX = 8
E_UNSUPPORTED = 9

PREC_FP32 = 0
PREC_BF16X3 = 1
PREC_BF16X2 = 2
PREC_BF16X1 = 3
PREC_FP16X2 = 4
PREC_FP8X5 = 5
PREC_AUTO = 6

MODE_SUM = 0
MODE_STACKED = 1

PRECISIONS = {
    "fp32": PREC_FP32,
    "bf16x3": PREC_BF16X3,
    "bf16x2": PREC_BF16X2,
    "bf16x1": PREC_BF16X1,
    "fp16x2": PREC_FP16X2,
    "fp8x5": PREC_FP8X5,
    "auto": PREC_AUTO,
}

_lock = threading.Lock()
_lib: C.CDLL | None = None

_p = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_u64 = C.c_uint64
_u32 = C.c_uint32
_f32 = C.c_float

_SIGNATURES = {
    "coherit_last_error": (C.c_char_p, []),
    "coherit_version": (C.c_int, []),
    "coherit_launch_count": (C.c_int64, []),
    "coherit_device_info": (C.c_int, [C.c_int, _p, _p, _p, _p]),
    "coherit_geno_create_packed": (
        C.c_int,
        [_p, _i64, _i32, _p, _p, _i32, C.c_int, C.c_int, _p, _p],
    ),
    "coherit_geno_create_synthetic": (
        C.c_int,
        [_i64, _i64, _p, _i32, _u64, _u32, C.c_int, _p, _p],
    ),
    "coherit_geno_create_bed": (
        C.c_int,
        [_p, _i64, _i64, _i64, _p, _i64, _p, _i32, C.c_int, _p, _p],
    ),
    "coherit_ldblock_records": (C.c_int, [_i64, _i64, _i32, _u64, _p, _p, _p, _p, _p, _p]),
    "coherit_geno_create_ldblock": (
        C.c_int,
        [_i64, _i64, _i32, _u64, _p, _p, _p, _p, _p, _p, _i32, C.c_int, _p, _p],
    ),
    "coherit_geno_destroy": (C.c_int, [_p]),
    "coherit_geno_info": (C.c_int, [_p, _p, _p, _p, _p, _p, _p, _p]),
    "coherit_geno_read_packed": (C.c_int, [_p, _i64, _i32, _p, _p]),
    "coherit_geno_compute_stats": (C.c_int, [_p, _i32, _p, _p, _p, _p, _p]),
    "coherit_geno_set_stats": (C.c_int, [_p, _i32, _p, _p, _p, _p]),
    "coherit_geno_release_stats": (C.c_int, [_p, _i32]),
    "coherit_geno_stats_summary": (C.c_int, [_p, _i32, _p, _p, _p, _p]),
    "coherit_geno_exact_diag": (C.c_int, [_p, _i32, _p, _p]),
    "coherit_geno_reserve": (C.c_int, [_p, _i32, _i32]),
    "coherit_geno_autotune": (C.c_int, [_p, _i32, _i32, _i32, _p, _p, _p, _p]),
    "coherit_mma_rate": (C.c_int, [_i32, _i32, _i32, _i32, _p, _p, _p]),
    "coherit_geno_set_launch": (C.c_int, [_p, _i32, _i32, _p]),
    "coherit_geno_kv": (
        C.c_int,
        [_p, _i32, _i32, _i32, _p, _i64, _i32, _p, _i32, _f32, _p, _p, _i64, _p],
    ),
    "coherit_geno_extract_columns": (C.c_int, [_p, _i32, _p, _i32, _p, _i64, _p]),
    "coherit_geno_kv_noalloc": (
        C.c_int,
        [_p, _i32, _i32, _i32, _p, _i64, _i32, _p, _i32, _f32, _p, _p, _i64, _p],
    ),
    "coherit_geno_kv_batched": (
        C.c_int,
        [_p, _i32, _p, _p, _i32, _p, _i64, _i32, _p, _p, _p, _i64, _p],
    ),
    "coherit_geno_xtv": (C.c_int, [_p, _i32, _i32, _p, _i64, _i32, _p, _p, _i64, _p]),
    "coherit_geno_zxb": (C.c_int, [_p, _i32, _i32, _p, _i64, _i32, _p, _i64, _p]),
    "coherit_geno_check": (C.c_int, [_p, _p]),
    "coherit_colreduce": (C.c_int, [_i32, _i64, _i32, _p, _i64, _p, _i64, _p, _p]),
    "coherit_pcg_state_update": (
        C.c_int,
        [_i64, _i32, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p, _p, _p, _p],
    ),
    "coherit_pcg_direction_update": (
        C.c_int,
        [_i64, _i32, _p, _i64, _p, _i64, _p, _p, _p, _p, _p, _p, _p],
    ),
    "coherit_lowrank_workspace_floats": (C.c_int, [_i64, _i32, _i32, _p]),
    "coherit_lowrank_apply": (
        C.c_int,
        [_i64, _i32, _i32, _p, _i64, _p, _i64, _f32, _p, _i64, _p, _i64, _p, _i64, _p],
    ),
    "coherit_selftest_mma": (C.c_int, [_i32, _p, _p]),
    "coherit_sparse_create_bed": (
        C.c_int,
        [_p, _i64, _i64, _i64, _p, _i64, C.c_int, _p, _p],
    ),
    "coherit_sparse_create_synthetic": (
        C.c_int,
        [_i64, _i64, _u64, _u32, _u32, _u32, C.c_int, _p, _p],
    ),
    "coherit_sparse_create_csc": (C.c_int, [_i64, _i64, _p, _p, _p, C.c_int, _p, _p]),
    "coherit_sparse_destroy": (C.c_int, [_p]),
    "coherit_sparse_info": (C.c_int, [_p, _p, _p, _p, _p, _p]),
    "coherit_sparse_stats": (C.c_int, [_p, _p, _p, _p, _p, _p, _p, _p]),
    "coherit_sparse_read_csc": (C.c_int, [_p, _p, _p, _p]),
    "coherit_sparse_set_stats": (C.c_int, [_p, _p, _p, _p]),
    "coherit_sparse_kv": (C.c_int, [_p, _p, _i64, _i32, C.c_double, _f32, _p, _i64, _p]),
    "coherit_sparse_xtv": (C.c_int, [_p, _p, _i64, _i32, C.c_double, _p, _i64, _p]),
    "coherit_sparse_extract_columns": (C.c_int, [_p, _p, _i32, _p, _i64, _p]),
    "coherit_sparse_exact_diag": (C.c_int, [_p, _p, _p]),
}


def library_path() -> Path:
    return build_ext.LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = build_ext.LIB_PATH
        if build_if_missing and build_ext.needs_build():
            build_ext.build()
        if not path.exists():
            raise RuntimeError(
                f"coherit_gb300 CUDA library not found at {path}; run "
                "`python -m coherit_gb300.build_ext` (nvcc with sm_103a) first"
            )
        lib = C.CDLL(str(path))
        for name, (restype, argtypes) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def last_error() -> str:
    lib = load()
    msg = lib.coherit_last_error()
    return msg.decode() if msg else ""


def check(status: int, what: str = "") -> None:
    if status == OK:
        return
    msg = last_error()
    text = f"{what}: {msg}" if what else msg
    if status == E_SHAPE:
        raise ValueError(text)
    if status == E_INDEX:
        raise IndexError(text)
    if status in (E_NONFINITE, E_NOT_CONVERGED):
        raise FloatingPointError(text)
    if status == E_OOM:
        raise MemoryError(text)
    raise RuntimeError(f"{text} (status {status})")


def ptr(t) -> int:
    """Device/host address of a torch tensor or numpy array (None -> 0)."""
    if t is None:
        return 0
    if hasattr(t, "data_ptr"):
        return int(t.data_ptr())
    return int(t.ctypes.data)


def stream_ptr(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)
