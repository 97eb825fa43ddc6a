"""SMILE host logic without a GPU: W file loading, validation, sidecar
metadata, bucket estimates, and the FP64 oracle's identity case."""
import json

import numpy as np
import pytest

from coherit_gb300 import smile_block_w as sm
from oracle import geno as og
from oracle import smile as osm


def test_weight_file_formats(tmp_path):
    W = np.arange(9, dtype=np.float64).reshape(3, 3)
    np.save(tmp_path / "a.npy", W)
    np.savez(tmp_path / "b.npz", w=W)
    np.savetxt(tmp_path / "c.csv", W, delimiter=",")
    np.savetxt(tmp_path / "d.txt", W)
    for name in ("a.npy", "b.npz", "c.csv", "d.txt"):
        np.testing.assert_array_equal(np.asarray(sm.load_weight_matrix(tmp_path / name)), W)
        assert sm.load_weight_matrix_shape(tmp_path / name) == (3, 3)
    np.savez(tmp_path / "two.npz", a=W, b=W)
    with pytest.raises(ValueError):
        sm.load_weight_matrix(tmp_path / "two.npz")
    (tmp_path / "a.json").write_text(json.dumps({"effective_rank": 2.5, "shape": [3, 3]}))
    assert sm.load_weight_matrix_metadata(tmp_path / "a.npy")["effective_rank"] == 2.5
    with pytest.raises(ValueError, match="Missing sidecar"):
        sm.load_weight_matrix_metadata(tmp_path / "d.txt", required=True)


def test_validate_and_effective_rank():
    with pytest.raises(ValueError, match="square"):
        sm.validate_weight_matrix(np.zeros((2, 3)))
    with pytest.raises(ValueError, match="non-finite"):
        sm.validate_weight_matrix(np.array([[1.0, np.nan], [0.0, 1.0]]))
    W = sm.validate_weight_matrix(np.eye(4, dtype=np.float64))
    assert W.dtype == np.float32 and W.flags.c_contiguous
    f = sm.SmileBlockWeightedOperator._effective_rank_contribution
    assert f(source=None, explicit_rank=3.0, width=4, block_name="W") == 3.0
    with pytest.raises(ValueError):
        f(source=None, explicit_rank=5.0, width=4, block_name="W")
    with pytest.raises(ValueError):
        f(source=None, explicit_rank=None, width=4, block_name="W")


def test_bucket_estimates():
    assert sm._bucket_width(500) == 512 and sm._bucket_width(513) == 1024
    assert sm.estimate_bucketed_w_device_cache_bytes([500, 500], 1e9) == 2 * 512 * 512 * 4
    assert sm.estimate_bucketed_w_device_cache_bytes([500], 100.0) == 0.0
    assert sm.default_w_device_cache_bytes(None) == 0.0
    assert sm.default_w_device_cache_bytes(1e10) == 0.35e10


def test_oracle_identity_blocks_equal_grm():
    codes = og.synth_codes(8, 60, np.arange(200))
    mean, inv, _ = og.stats(codes)
    Z = osm.standardized(codes, mean, inv)
    k = osm.SmileKernel.identity(Z, 64)
    eff = float(np.count_nonzero(inv > 0))
    V = np.random.default_rng(0).normal(size=(60, 3))
    ref = og.kv_f64(codes, mean, inv, V, comp_scale=[1.0 / k.c])
    np.testing.assert_allclose(k.kv(V), ref, rtol=1e-10, atol=1e-12)
    assert abs(k.c - eff) < 1e-4 * eff
    np.testing.assert_allclose(k.diag_mean(), 1.0, rtol=1e-12)
