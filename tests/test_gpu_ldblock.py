"""Block-LD genotypes of the 8-component workload, generated on the device,
against the numpy twin of the generator (bit-exact codes), and an 8-component
fit on them (4 MAF bins x 2 LD-score halves as arbitrary variant groups)
against the FP64 oracle fit on the same probes: |delta h2| < 1e-3."""
import ctypes as C

import numpy as np
import pytest
import torch

from coherit_gb300 import _lib, synth
from coherit_gb300.geno_stream import GenoBlockStreamer, LDBlockSource
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter
from oracle import geno as og
from oracle import reml as oreml

pytestmark = pytest.mark.gpu


def _decode_records(rec, n):
    """SNP-major BED records (m, ceil(n/4)) -> counts (n, m)."""
    lut = np.array([2, 0, 1, 0], np.uint8)  # BED 0,1,2,3 -> 2, missing(none), 1, 0
    r = np.asarray(rec)
    codes = np.stack([lut[(r >> (2 * t)) & 3] for t in range(4)], axis=2)
    return codes.reshape(r.shape[0], -1)[:, :n].T


def test_device_records_match_numpy_twin(cuda):
    seed, n, m, block = 17, 333, 1000, 200
    thr, rho, sfac, quant, _ = tables = synth.ld_tables(seed, m, block=block)
    td = [torch.as_tensor(a, device=cuda) for a in (thr, rho, sfac, quant)]
    rec = torch.empty((m, (n + 3) // 4), dtype=torch.uint8, device=cuda)
    lib = _lib.load()
    _lib.check(lib.coherit_ldblock_records(n, m, block, seed, *(t.data_ptr() for t in td),
                                           rec.data_ptr(), _lib.stream_ptr()))
    got = _decode_records(rec.cpu().numpy(), n)
    want = synth.ld_block_codes(seed, n, m, block=block, tables=tables)
    np.testing.assert_array_equal(got, want)


def test_resident_matrix_in_cache_order(cuda):
    seed, n, m = 5, 300, 1200
    src = LDBlockSource(n, m, seed=seed)
    codes = synth.ld_block_codes(seed, n, m, tables=src.tables)
    groups = synth.maf_ld_partition(src.tables[4], synth.block_ld_scores(codes))
    st = GenoBlockStreamer(src, component_variant_indices=groups, precision="bf16x3")
    try:
        order = np.concatenate(groups)
        host = np.empty((n, (m + 3) // 4), np.uint8)
        _lib.check(_lib.load().coherit_geno_read_packed(st.handle, 0, m, host.ctypes.data,
                                                        _lib.stream_ptr()))
        np.testing.assert_array_equal(og.unpack_block(host, m), codes[:, order])
        mean, inv, _ = og.stats(codes[:, order])
        np.testing.assert_array_equal(st._means_host, mean)
        np.testing.assert_array_equal(st._inv_sds_host, inv)
    finally:
        st.close()


def test_partition_from_device_ld_scores(cuda):
    seed, m, n_ld = 23, 1400, 512
    groups, tables = synth.ld_partition_device(seed, m, n_ld=n_ld, device=cuda)
    assert len(groups) == 8
    np.testing.assert_array_equal(np.sort(np.concatenate(groups)), np.arange(m))
    codes = synth.ld_block_codes(seed, n_ld, m, tables=tables)
    ld = synth.block_ld_scores(codes)
    maf = tables[4]
    for b in range(4):
        lo, hi = groups[2 * b], groups[2 * b + 1]
        # LD scores in FP32 on the device vs FP64 here: the halves split at
        # the same place up to ties within 1e-4.
        assert ld[lo].max() <= ld[hi].min() + 1e-4
        if b:
            prev = np.concatenate(groups[2 * b - 2: 2 * b])
            assert maf[prev].max() <= maf[np.concatenate([lo, hi])].min()


def test_eight_component_fit_matches_oracle(cuda):
    seed, n, m = 31, 700, 3200
    src = LDBlockSource(n, m, seed=seed)
    codes = synth.ld_block_codes(seed, n, m, tables=src.tables)
    groups = synth.maf_ld_partition(src.tables[4], synth.block_ld_scores(codes))
    h2s = synth.dirichlet_h2(seed, 8, total=0.4)
    y, X = synth.partitioned_phenotype(codes, groups, h2s, seed=seed, n_causal_per=40, n_covar=2)
    st = GenoBlockStreamer(src, component_variant_indices=groups, precision="bf16x3")
    try:
        probes = np.random.default_rng(3).choice([-1.0, 1.0], size=(n, 16))
        cfg = FitConfig(slq_samples=16, slq_m=14, reml_pcg_tol=1e-5, minq_iter=15,
                        max_pcg_iters=1000, slq_mode="raw")
        res = InfinitesimalREMLFitter(cfg, [st]).fit_infinitesimal(
            y, X, slq_probes=torch.as_tensor(probes, dtype=torch.float32))
        order = np.concatenate(groups)
        mean, inv = st._means_host, st._inv_sds_host
        Z = og.diff_f64(codes[:, order], mean) * inv.astype(np.float64)[None, :]
        Ks, pos = [], 0
        for g, grp in enumerate(groups):
            Zg = Z[:, pos:pos + grp.size]
            Ks.append(Zg @ Zg.T / float(st._component_eff_m_host[g]))
            pos += grp.size
        yo, _, _ = oreml.standardize(y)
        atoms = st._component_mean_diag_atoms_host.astype(np.float64)
        ctx = oreml.Context(yo, [(lambda v, K=K: K @ v) for K in Ks], X, diag_atoms=atoms,
                            slq_probes=probes, slq_m=14, pcg_tol=1e-5, maxiter=1000)
        po, _, _ = oreml.fit(ctx, minq_iter=15)
        h2_ref = oreml.heritability(po, 8, atoms)
        assert abs(res.heritability - h2_ref) < 1e-3, (res.heritability, h2_ref)
    finally:
        st.close()
