"""Host-side checks of the rare-variant path that need no GPU: shard
argument validation of the kv_impl shims and the sparse C ABI's validation
of host entry lists (both reject before touching a device)."""
import ctypes as C

import numpy as np
import pytest

from coherit_gb300 import _lib, kv_impl


def test_shard_arrays_must_agree():
    with pytest.raises(ValueError, match="one length"):
        kv_impl._TransientSparse(10, 3, np.zeros(3), np.ones(3), [0, 1], [0], [1], None)
    with pytest.raises(ValueError, match="ascending"):
        kv_impl._TransientSparse(10, 3, np.zeros(3), np.ones(3), [0, 1], [2, 1],
                                 np.asarray([1, 1], np.int8), None)
    with pytest.raises(ValueError, match="ascending"):
        kv_impl._TransientSparse(10, 3, np.zeros(3), np.ones(3), [0], [3],
                                 np.asarray([1], np.int8), None)
    with pytest.raises(ValueError, match="m=3"):
        kv_impl._TransientSparse(10, 3, np.zeros(2), np.ones(3), [0], [0],
                                 np.asarray([1], np.int8), None)


@pytest.mark.parametrize("case,status", [
    ("offset0", _lib.E_SHAPE),
    ("decreasing", _lib.E_SHAPE),
    ("row", _lib.E_INDEX),
    ("value", _lib.E_SHAPE),
])
def test_csc_entry_lists_validated_before_device_use(case, status):
    lib = _lib.load()
    col_off = np.asarray([0, 2, 3], np.int64)
    rows = np.asarray([0, 4, 2], np.int32)
    vals = np.asarray([1, 2, 3], np.int8)
    if case == "offset0":
        col_off = np.asarray([1, 2, 3], np.int64)
    elif case == "decreasing":
        col_off = np.asarray([0, 3, 2], np.int64)
    elif case == "row":
        rows = np.asarray([0, 9, 2], np.int32)
    elif case == "value":
        vals = np.asarray([1, 0, 3], np.int8)
    h = C.c_void_p()
    rc = lib.coherit_sparse_create_csc(5, 2, col_off.ctypes.data, rows.ctypes.data,
                                       vals.ctypes.data, 0, None, C.byref(h))
    assert rc == status
    assert not h
    assert _lib.last_error()


def test_null_sparse_handle_is_rejected():
    lib = _lib.load()
    assert lib.coherit_sparse_info(None, None, None, None, None, None) == _lib.E_CLOSED
    assert lib.coherit_sparse_kv(None, None, 1, 1, 1.0, 0.0, None, 1, None) == _lib.E_CLOSED
