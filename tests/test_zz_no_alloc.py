"""coherit_geno_kv_noalloc (workspace in a fixed static device array) against
coherit_geno_kv on the same handle and inputs (GPU).

Tolerance: every output column within 1e-5 relative (2-norm) of
coherit_geno_kv's.  Both run the same kernels; they differ only in the order
of FP64 atomic additions.  Each case makes two fixed-scratch calls in a row
with different right-hand sides and checks that the handle's device
footprint (which includes its growable workspace) does not change.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from coherit_gb300 import _lib

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _create(n, m, comps=None, missing_q24=0, seed=5):
    lib = _lib.load()
    h = C.c_void_p()
    arr = None if comps is None else np.asarray(comps, dtype=np.int32)
    _lib.check(lib.coherit_geno_create_synthetic(
        n, m, None if arr is None else arr.ctypes.data, 1 if arr is None else arr.size, seed,
        missing_q24, 0, _lib.stream_ptr(), C.byref(h)), "create")
    return h


def _device_bytes(h):
    vals = [C.c_int64() for _ in range(6)]
    g = C.c_int32()
    _lib.check(_lib.load().coherit_geno_info(h, C.byref(vals[0]), C.byref(vals[1]),
                                             C.byref(vals[2]), C.byref(vals[3]), C.byref(g),
                                             C.byref(vals[4]), C.byref(vals[5])), "info")
    return vals[5].value


def _apply(fn_name, h, V, G, mode=0, precision=1, scale=None, theta_e=None):
    n, k = V.shape
    out = torch.empty((G if mode == 1 else 1, n, k), dtype=torch.float32, device=V.device)
    sc = np.ones(G, dtype=np.float32) if scale is None else np.asarray(scale, np.float32)
    fn = getattr(_lib.load(), fn_name)
    _lib.check(fn(h, 0, mode, precision, V.data_ptr(), k, k, sc.ctypes.data,
                  0 if theta_e is None else 1, 0.0 if theta_e is None else theta_e, None,
                  out.data_ptr(), k, _lib.stream_ptr()), fn_name)
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


def _col_rel(out, ref):
    out = out.reshape(-1, out.shape[-1])
    ref = ref.reshape(-1, ref.shape[-1])
    num = np.linalg.norm(out - ref, axis=0)
    return float(np.max(num / np.maximum(np.linalg.norm(ref, axis=0), 1e-300)))


def _check_pair(h, G, k, mode, precision, scale=None, theta_e=None, seed=0):
    gen = torch.Generator(device="cuda").manual_seed(seed)
    n = _n_of(h)
    V1 = torch.randn((n, k), generator=gen, device="cuda")
    V2 = torch.randn((n, k), generator=gen, device="cuda")
    before = _device_bytes(h)
    a1 = _apply("coherit_geno_kv_noalloc", h, V1, G, mode, precision, scale, theta_e)
    a2 = _apply("coherit_geno_kv_noalloc", h, V2, G, mode, precision, scale, theta_e)
    assert _device_bytes(h) == before
    r1 = _apply("coherit_geno_kv", h, V1, G, mode, precision, scale, theta_e)
    r2 = _apply("coherit_geno_kv", h, V2, G, mode, precision, scale, theta_e)
    assert _col_rel(a1, r1) < TOL
    assert _col_rel(a2, r2) < TOL
    assert np.all(np.isfinite(a1)) and np.all(np.isfinite(a2))
    return (V1, a1), (V2, a2)


def _n_of(h):
    n = C.c_int64()
    _lib.check(_lib.load().coherit_geno_info(h, C.byref(n), None, None, None, None, None, None))
    return n.value


def test_noalloc_sum_with_missing_matches_kv(cuda):
    """Both fixed-scratch calls are also checked against the FP64 oracle
    (sum over two components with missing genotypes and theta_e), so a fault
    shared by both entry points (launch sequence, workspace offsets) shows."""
    from oracle import geno as og

    n, m, miss_q24 = 3000, 7000, int(0.01 * (1 << 24))
    h = _create(n, m, comps=[3000, 4000], missing_q24=miss_q24)
    try:
        assert _device_bytes(h) > 0
        scale = [1 / 3000.0, 1 / 4000.0]
        calls = _check_pair(h, 2, 20, 0, 1, scale=scale, theta_e=0.7, seed=1)
        codes = og.synth_codes(5, n, np.arange(m), missing_q24=miss_q24)
        mean, inv, _ = og.stats(codes)
        comp = np.repeat([0, 1], [3000, 4000])
        for V, got in calls:
            ref = og.kv_f64(codes, mean, inv, V.cpu().numpy(), comp_of_snp=comp,
                            comp_scale=scale, n_components=2, theta_e=0.7)
            assert _col_rel(got, ref) < TOL
    finally:
        _lib.load().coherit_geno_destroy(h)


def test_noalloc_stacked_wide_and_bf16x1_match_kv(cuda):
    h = _create(2500, 5000, comps=[2000, 3000])
    try:
        # 200 columns: two column blocks per call at bf16x3.
        _check_pair(h, 2, 200, 1, 1, scale=[0.5, 2.0], seed=2)
        _check_pair(h, 2, 33, 0, 3, seed=3)
        _check_pair(h, 2, 40, 0, 4, seed=4)
        _check_pair(h, 2, 24, 1, 5, seed=5)
    finally:
        _lib.load().coherit_geno_destroy(h)


def test_noalloc_rejects_oversized_and_fp32(cuda):
    lib = _lib.load()
    # 200k SNPs x 112 columns x 3 split terms of BF16 S tiles alone exceed 64 MiB.
    h = _create(256, 200_000)
    try:
        V = torch.zeros((256, 112), device="cuda")
        out = torch.empty_like(V)
        sc = np.ones(1, np.float32)
        st = lib.coherit_geno_kv_noalloc(h, 0, 0, 1, V.data_ptr(), 112, 112, sc.ctypes.data, 0,
                                         0.0, None, out.data_ptr(), 112, _lib.stream_ptr())
        assert st == _lib.E_SHAPE
        assert b"fixed scratch" in lib.coherit_last_error()
        st = lib.coherit_geno_kv_noalloc(h, 0, 0, 0, V.data_ptr(), 112, 16, sc.ctypes.data, 0,
                                         0.0, None, out.data_ptr(), 112, _lib.stream_ptr())
        assert st == _lib.E_UNSUPPORTED
        # A narrow block of the same matrix fits and still allocates nothing.
        before = _device_bytes(h)
        st = lib.coherit_geno_kv_noalloc(h, 0, 0, 1, V.data_ptr(), 112, 16, sc.ctypes.data, 0,
                                         0.0, None, out.data_ptr(), 112, _lib.stream_ptr())
        assert st == _lib.OK
        torch.cuda.synchronize()
        assert _device_bytes(h) == before
        assert float(out[:, :16].abs().max()) == 0.0
    finally:
        lib.coherit_geno_destroy(h)
