"""The GWAS oracle against direct least squares of y on [X, z_j] (CPU)."""
import numpy as np
import pytest

from oracle import geno as og
from oracle import gwas as ogw
from oracle import smile as osm


def test_fwl_statistics_equal_direct_least_squares():
    rng = np.random.default_rng(0)
    n, m = 300, 40
    codes = og.synth_codes(4, n, np.arange(m), missing_q24=int(0.02 * (1 << 24)))
    mean, inv, cnt = og.stats(codes)
    Z = osm.standardized(codes, mean, inv)
    X = np.column_stack([np.ones(n), rng.normal(size=(n, 2))])
    y = rng.normal(size=n) + Z[:, 3]
    counts = np.sum(codes != 3, axis=0)
    out = ogw.scan(Z, counts, inv, y, X)
    for j in range(m):
        if inv[j] == 0:
            continue
        A = np.column_stack([X, Z[:, j]])
        coef, res, *_ = np.linalg.lstsq(A, y, rcond=None)
        resid = y - A @ coef
        sigma2 = resid @ resid / (n - A.shape[1])
        cov = sigma2 * np.linalg.inv(A.T @ A)
        np.testing.assert_allclose(out["beta_std"][j], coef[-1], rtol=1e-5, atol=1e-9)
        np.testing.assert_allclose(out["se_std"][j], np.sqrt(cov[-1, -1]), rtol=1e-4)


def test_gwas_rejects_fitters_with_rare_variant_streamers(tmp_path):
    """gwas.py:77-86: sparse genotype inputs are not scanned."""
    import types

    from coherit_gb300.gwas import run_continuous_gwas

    fake = types.SimpleNamespace(_has_sparse=True, streamers=[object()], _n_dense_streamers=1)
    with pytest.raises(ValueError, match="dense genotype inputs only"):
        run_continuous_gwas(fake, np.zeros(4), out_prefix=str(tmp_path / "g"))
    empty = types.SimpleNamespace(_has_sparse=False, streamers=[], _n_dense_streamers=0)
    with pytest.raises(ValueError, match="at least one dense"):
        run_continuous_gwas(empty, np.zeros(4), out_prefix=str(tmp_path / "g"))
