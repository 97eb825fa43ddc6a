"""Marginal GWAS scan on the GPU operator against the FP64 oracle.

Tolerances: beta, se, t within 1e-5 of each statistic's scale (its largest
magnitude over the SNPs: the bf16x3 X^T V pass is accurate relative to a
column's norm, so near-zero effects carry the same absolute error as the
others); p-values within 1e-4 relative.  The TSV output has the reference's
columns and one row per variant."""
import numpy as np
import pytest

from coherit_gb300 import synth
from coherit_gb300.bed import write_bed
from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
from coherit_gb300.gwas import GWAS_HEADER, marginal_scan, run_continuous_gwas
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter
from oracle import geno as og
from oracle import gwas as ogw
from oracle import smile as osm

pytestmark = pytest.mark.gpu


def _close(a, b, rtol, scaled=True):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), ok)
    atol = rtol * np.max(np.abs(b[ok])) if scaled else 0.0
    np.testing.assert_allclose(a[ok], b[ok], rtol=0 if scaled else rtol, atol=atol)


def test_marginal_scan_matches_oracle(cuda):
    n, m = 1500, 2000
    miss = 0.01
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=91, missing_rate=miss))
    codes = og.synth_codes(91, n, np.arange(m), missing_q24=synth.missing_rate_q24(miss))
    y, X, _, _ = synth.phenotype(91, n, m, h2=0.3, n_causal=50, n_covar=3,
                                 missing_q24=synth.missing_rate_q24(miss))
    got = marginal_scan(st, y, X)
    Z = osm.standardized(codes, st._means_host, st._inv_sds_host)
    ref = ogw.scan(Z, st._count_host, st._inv_sds_host, y, X)
    assert got["dof"] == ref["dof"] == n - 4 - 1
    for key in ("beta_std", "se_std", "t", "beta", "se"):
        _close(got[key], ref[key], 1e-5)
    _close(got["p"], ref["p"], 1e-4, scaled=False)
    # Without covariates the intercept alone is projected out.
    got0 = marginal_scan(st, y)
    ref0 = ogw.scan(Z, st._count_host, st._inv_sds_host, y, np.ones((n, 1)))
    _close(got0["t"], ref0["t"], 1e-5)


def test_run_continuous_gwas_writes_tsv(cuda, tmp_path):
    n, m = 600, 700
    codes = og.synth_codes(92, n, np.arange(m))
    prefix = str(tmp_path / "g")
    write_bed(prefix, codes.astype(np.int16))
    st = GenoBlockStreamer(bed_prefix=prefix)
    y = np.random.default_rng(0).normal(size=n).astype(np.float32)
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=0), [st])
    summary = run_continuous_gwas(fitter, y, None, out_prefix=str(tmp_path / "out" / "scan"))
    lines = open(summary.out_path).read().splitlines()
    assert lines[0] + "\n" == GWAS_HEADER
    assert len(lines) == m + 1 and summary.n_variants == m and summary.dof == n - 2
    stats = marginal_scan(st, y)
    row = lines[1 + 123].split("\t")
    assert row[5] == "rs123" and int(row[11]) == n
    np.testing.assert_allclose(float(row[16]), stats["t"][123], rtol=1e-6)
