"""Host side of the marginal GWAS scan on CPU, through a numpy streamer.

``marginal_scan`` reaches the device only through ``streamer.xtv``; a
streamer whose ``xtv`` is the dense FP64 product Z^T V on CPU runs the rest
of the scan (covariate basis, per-SNP statistics, p-values) and the writer
of the reference's TSV rows and metadata (gwas.py:70-247, gwas_io.py:8-31).
Statistics are compared with the oracle scan on the same Z.
"""
import json
import types

import numpy as np
import pytest
import torch

from coherit_gb300 import bed, gwas
from oracle import geno as og
from oracle import gwas as ogw
from oracle import smile as osm


class _DenseStreamer:
    """The attributes and the X^T V of a dense streamer, computed on the host."""

    def __init__(self, codes, bed_prefix=None):
        self.codes = codes
        self.n, self.m = codes.shape
        mean, inv, cnt = og.stats(codes)
        self._means_host, self._inv_sds_host = mean, inv
        self._count_host = np.asarray(cnt, np.int64)
        self.Z = osm.standardized(codes, mean, inv)
        self.dev = torch.device("cpu")
        self.bed_prefix = bed_prefix

    def xtv(self, V, normalize=False):
        assert not normalize
        return torch.as_tensor(self.Z.T @ V.double().numpy())


def _codes(seed, n, m, monomorphic=()):
    codes = og.synth_codes(seed, n, np.arange(m), missing_q24=int(0.03 * (1 << 24)))
    for j in monomorphic:
        codes[:, j] = 1
    return codes


def _check_against_oracle(st, y, X, out):
    ref = ogw.scan(st.Z, st._count_host, st._inv_sds_host, y,
                   np.ones((st.n, 1)) if X is None else X)
    ok = st._inv_sds_host > 0
    for key in ("beta", "se", "beta_std", "se_std", "t"):
        np.testing.assert_allclose(out[key][ok], ref[key][ok], rtol=1e-5, atol=1e-9)
        assert np.all(np.isnan(out[key][~ok]))
    np.testing.assert_allclose(out["p"][ok], ref["p"][ok], rtol=1e-4, atol=1e-12)
    assert out["dof"] == ref["dof"]


@pytest.mark.parametrize("covar", ["none", "full_rank", "rank_deficient", "vector"])
def test_marginal_scan_equals_oracle(covar):
    rng = np.random.default_rng(1)
    n, m = 120, 30
    st = _DenseStreamer(_codes(2, n, m, monomorphic=(4,)))
    y = (rng.normal(size=n) + st.Z[:, 7]).astype(np.float32)
    X = None
    if covar == "full_rank":
        X = np.column_stack([np.ones(n), rng.normal(size=(n, 3))])
    elif covar == "rank_deficient":
        a = rng.normal(size=n)
        X = np.column_stack([np.ones(n), a, 2 * a])
    elif covar == "vector":
        X = np.ones(n)
    out = gwas.marginal_scan(st, y, X)
    Xo = None if X is None else (X[:, None] if X.ndim == 1 else X)
    _check_against_oracle(st, y.astype(np.float64), Xo, out)
    expected_rank = {"none": 1, "full_rank": 4, "rank_deficient": 2, "vector": 1}[covar]
    assert out["rank"] == expected_rank and out["dof"] == n - expected_rank - 1
    assert out["p"][7] < 1e-6
    np.testing.assert_allclose(out["af"], st._means_host / 2.0)


def test_marginal_scan_contract_errors():
    st = _DenseStreamer(_codes(3, 10, 5))
    with pytest.raises(ValueError, match="Sample-size mismatch"):
        gwas.marginal_scan(st, np.zeros(9))
    with pytest.raises(ValueError, match="Covariate row mismatch"):
        gwas.marginal_scan(st, np.ones(10), np.ones((9, 2)))
    with pytest.raises(ValueError, match="degrees of freedom"):
        gwas.marginal_scan(st, np.arange(10.0), np.random.default_rng(0).normal(size=(10, 9)))
    st._count_host = None
    with pytest.raises(ValueError, match="non-missing counts"):
        gwas.marginal_scan(st, np.arange(10.0))


def test_run_continuous_gwas_writes_reference_rows(tmp_path, monkeypatch):
    monkeypatch.setattr(gwas, "_WRITE_CHUNK_ROWS", 7)   # rows written in several chunks
    rng = np.random.default_rng(5)
    n = 64
    streamers = []
    for i, m in enumerate((19, 11)):
        codes = _codes(10 + i, n, m, monomorphic=(2,) if i == 0 else ())
        prefix = str(tmp_path / f"chr{i + 1}")
        bed.write_bed(prefix, np.where(codes == 3, -1, codes.astype(np.int8)))
        streamers.append(_DenseStreamer(codes, bed_prefix=prefix + ".bed"))
    fitter = types.SimpleNamespace(streamers=streamers, _n_dense_streamers=2, _has_sparse=False)
    y = rng.normal(size=n).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.normal(size=n)])
    summ = gwas.run_continuous_gwas(fitter, y, X, out_prefix=str(tmp_path / "out" / "trait"))
    assert (summ.n_samples, summ.n_variants, summ.dof, summ.n_covar_cols) == (n, 30, n - 3, 2)
    lines = open(summ.out_path).read().splitlines()
    assert lines[0] + "\n" == gwas.GWAS_HEADER
    rows = [r.split("\t") for r in lines[1:]]
    assert len(rows) == 30 and all(len(r) == 18 for r in rows)
    g = 0
    for ci, st in enumerate(streamers):
        out = gwas.marginal_scan(st, y, X)
        for li in range(st.m):
            r = rows[g]
            assert r[:10] == [str(ci), f"chr{ci + 1}", str(g), str(li), "1", f"rs{li}", "0",
                              str(li + 1), "A", "C"]
            assert int(r[11]) == int(st._count_host[li])
            for col, key in zip(range(12, 18), ("beta", "se", "beta_std", "se_std", "t", "p")):
                v = float(r[col])
                if np.isnan(out[key][li]):
                    assert r[col] == "nan"
                else:
                    assert v == pytest.approx(float(out[key][li]), rel=1e-7, abs=1e-300)
            assert float(r[10]) == pytest.approx(float(st._means_host[li]) / 2, rel=1e-7)
            g += 1
    meta = json.load(open(summ.metadata_path))
    assert meta["n_variants"] == 30 and meta["dof"] == n - 3 and meta["rank_covar"] == 2
    assert meta["files"] == {"gwas": summ.out_path}
    assert [c["n_variants"] for c in meta["components"]] == [19, 11]
    assert [c["component_name"] for c in meta["components"]] == ["chr1", "chr2"]


def test_run_continuous_gwas_metadata_errors(tmp_path):
    codes = _codes(20, 16, 5)
    st = _DenseStreamer(codes)
    fitter = types.SimpleNamespace(streamers=[st], _n_dense_streamers=1, _has_sparse=False)
    with pytest.raises(ValueError, match="sidecar"):
        gwas.run_continuous_gwas(fitter, np.arange(16.0), out_prefix=str(tmp_path / "a"))
    with pytest.raises(ValueError, match="out_prefix"):
        gwas.run_continuous_gwas(fitter, np.arange(16.0), out_prefix="")
    prefix = str(tmp_path / "short")
    bed.write_bed(prefix, codes[:, :4].astype(np.int8))     # .bim with 4 of the 5 SNPs
    st.bed_prefix = prefix
    with pytest.raises(RuntimeError, match="count mismatch"):
        gwas.run_continuous_gwas(fitter, np.arange(16.0), out_prefix=str(tmp_path / "b"))
    with open(prefix + ".bim", "w") as f:
        f.write("1 rs0 0\n")
    with pytest.raises(ValueError, match="fewer than 6"):
        gwas.run_continuous_gwas(fitter, np.arange(16.0), out_prefix=str(tmp_path / "c"))


def test_marginal_scan_requires_host_statistics():
    """gwas.py:92-93, :163-164 of the reference."""
    st = _DenseStreamer(_codes(4, 12, 6))
    st._means_host = None
    with pytest.raises(ValueError, match="keep_host_stats=True"):
        gwas.marginal_scan(st, np.arange(12.0))
    st = _DenseStreamer(_codes(4, 12, 6))
    st._count_host = st._count_host[:5]
    with pytest.raises(RuntimeError, match="count vector length"):
        gwas.marginal_scan(st, np.arange(12.0))
