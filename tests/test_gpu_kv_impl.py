"""kv_impl entry points with the reference signatures (resident and foreign pop_block)."""
import numpy as np
import pytest
import torch

from coherit_gb300 import kv_impl, synth
from coherit_gb300.geno_stream import GenoBlockStreamer, SyntheticSource
from oracle import geno as og

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64).reshape(len(a), -1)
    b = np.asarray(b, np.float64).reshape(len(b), -1)
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


def _setup(n=300, m=900, seed=41, miss=0.02, call_width=256):
    st = GenoBlockStreamer(SyntheticSource(n, m, seed=seed, missing_rate=miss),
                           call_width=call_width, precision="bf16x3")
    codes = og.synth_codes(seed, n, np.arange(m), missing_q24=synth.missing_rate_q24(miss))
    return st, codes


def test_kv_impl_streamed_resident_and_foreign_blocks(cuda):
    st, codes = _setup()
    V = torch.randn(st.n, 3, device=cuda)
    args = (V, st._true_widths_dev, st._means_by_call, st._inv_by_call, st._eff_m_const)
    kw = dict(n=st.n, n_calls=st._n_calls)
    a = kv_impl.kv_impl_streamed(*args, pop_block=st._pop_cached, **kw)
    blocks = [st._pop_cached(c) for c in range(st._n_calls)]
    b = kv_impl.kv_impl_streamed(*args, pop_block=lambda c: blocks[c], **kw)
    ref = og.kv_f64(codes, st._means_host, st._inv_sds_host, V.cpu().numpy(),
                    comp_scale=[1 / float(st._eff_m_const)])
    assert rel(a.cpu(), ref) < TOL
    assert rel(b.cpu(), ref) < TOL
    v1 = kv_impl.kv_impl_streamed(V[:, 0], *args[1:], pop_block=st._pop_cached, normalize=False, **kw)
    assert v1.shape == (st.n,)


def test_xtv_and_zxb_streamed(cuda):
    st, codes = _setup()
    V = torch.randn(st.n, 2, device=cuda)
    out = kv_impl.xtv_impl_streamed(V, st.m, st._snp_starts_dev, st._true_widths_dev,
                                    st._means_by_call, st._inv_by_call, n_calls=st._n_calls,
                                    pop_block=st._pop_cached, normalize=True,
                                    eff_m=st._eff_m_const)
    ref = og.xtv_f64(codes, st._means_host, st._inv_sds_host, V.cpu().numpy()) / float(st._eff_m_const)
    assert rel(out.cpu(), ref) < TOL
    with pytest.raises(ValueError):
        kv_impl.xtv_impl_streamed(V, st.m, st._snp_starts_dev, st._true_widths_dev,
                                  st._means_by_call, st._inv_by_call, n_calls=st._n_calls,
                                  pop_block=st._pop_cached, normalize=True)
    W = st._max_unpack_width
    b = np.zeros((st._n_calls, W), np.float32)
    flat = np.random.default_rng(0).normal(size=st.m).astype(np.float32)
    for c in range(st._n_calls):
        s0, w = int(st._call_snp_starts[c]), int(st._call_true_widths[c])
        b[c, :w] = flat[s0:s0 + w]
    comp_ids = np.arange(st._n_calls) % 2
    total, comps = kv_impl.zxb_impl_streamed(
        torch.as_tensor(b, device=cuda), st._true_widths_dev, st._means_by_call, st._inv_by_call,
        n=st.n, n_calls=st._n_calls, pop_block=st._pop_cached, component_ids=comp_ids,
        n_components=2)
    ref = og.zxb_f64(codes, st._means_host, st._inv_sds_host, flat)
    assert rel(total.cpu()[:, None], ref[:, None]) < TOL
    assert rel((comps[0] + comps[1]).cpu()[:, None], ref[:, None]) < TOL
    with pytest.raises(ValueError):
        kv_impl.zxb_impl_streamed(torch.as_tensor(b[:1], device=cuda), st._true_widths_dev,
                                  st._means_by_call, st._inv_by_call, n=st.n, n_calls=st._n_calls,
                                  pop_block=st._pop_cached)


def test_multi_streamer_weighted_and_stacked(cuda):
    st1, c1 = _setup(seed=43)
    st2, c2 = _setup(seed=47)
    V = torch.randn(st1.n, 2, device=cuda)
    theta = torch.tensor([0.3, 0.6])
    hv = kv_impl.kv_impl_multi_streamed_weighted(V, [st1, st2], [], theta, theta_e=0.2)
    e1, e2 = float(st1._eff_m_const), float(st2._eff_m_const)
    Vn = V.cpu().numpy()
    r1 = og.kv_f64(c1, st1._means_host, st1._inv_sds_host, Vn, comp_scale=[0.3 / e1])
    r2 = og.kv_f64(c2, st2._means_host, st2._inv_sds_host, Vn, comp_scale=[0.6 / e2])
    assert rel(hv.cpu(), r1 + r2 + 0.2 * Vn) < TOL
    stacked = kv_impl.kv_impl_multi_streamed_stacked(V, [st1, st2], [])
    assert stacked.shape == (2, st1.n, 2)
    assert rel(stacked[0].cpu(), r1 / 0.3) < TOL


def _b_rows(st, flat):
    b = np.zeros((st._n_calls, st._max_unpack_width), np.float32)
    for c in range(st._n_calls):
        s0, w = int(st._call_snp_starts[c]), int(st._call_true_widths[c])
        b[c, :w] = flat[s0:s0 + w]
    return b


def test_zxb_same_stream_multi_and_multi_streamed(cuda):
    st, codes = _setup()
    rng = np.random.default_rng(3)
    flats = rng.normal(size=(3, st.m)).astype(np.float32)
    stack = np.stack([_b_rows(st, f) for f in flats])
    blocks = [st._pop_cached(c) for c in range(st._n_calls)]
    refs = [og.zxb_f64(codes, st._means_host, st._inv_sds_host, f) for f in flats]
    for pop in (st._pop_cached, lambda c: blocks[c]):
        total, comps = kv_impl.zxb_impl_same_stream_multi(
            torch.as_tensor(stack, device=cuda), st._true_widths_dev, st._means_by_call,
            st._inv_by_call, n=st.n, n_calls=st._n_calls, pop_block=pop)
        assert len(comps) == 3
        for g in range(3):
            assert rel(comps[g].cpu()[:, None], refs[g][:, None]) < TOL
        assert rel(total.cpu()[:, None], sum(refs)[:, None]) < TOL
    st2, codes2 = _setup(seed=53)
    flat2 = rng.normal(size=st2.m).astype(np.float32)
    plan = [(0, c) for c in range(st._n_calls)] + [(1, c) for c in range(st2._n_calls)]
    total, comps = kv_impl.zxb_impl_multi_streamed(
        [torch.as_tensor(stack[0], device=cuda), _b_rows(st2, flat2)], [st, st2], plan)
    ref2 = og.zxb_f64(codes2, st2._means_host, st2._inv_sds_host, flat2)
    assert rel(comps[0].cpu()[:, None], refs[0][:, None]) < TOL
    assert rel(comps[1].cpu()[:, None], ref2[:, None]) < TOL
    assert rel(total.cpu()[:, None], (refs[0] + ref2)[:, None]) < TOL
    # Calls left out of the plan contribute nothing.
    part = kv_impl.zxb_impl_multi_streamed([stack[0]], [st], [(0, 0)])[1][0]
    only0 = flats[0].copy()
    only0[int(st._call_true_widths[0]):] = 0.0
    ref0 = og.zxb_f64(codes, st._means_host, st._inv_sds_host, only0)
    assert rel(part.cpu()[:, None], ref0[:, None]) < TOL


def test_snp_weighted_resident_foreign_and_streamer(cuda):
    """Z diag(w) Z^T V / denom (kv_impl.py:139-160, :329-379) through the
    streamer's resident path, a foreign pop_block and the streamer method,
    against the FP64 oracle with the same per-SNP weights."""
    st, codes = _setup(seed=59)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.05, 2.0, size=st.m).astype(np.float32)
    w[::7] = 0.0
    wb = _b_rows(st, w)
    denom = 137.25
    V = torch.randn(st.n, 5, device=cuda)
    ref = og.kv_f64(codes, st._means_host, st._inv_sds_host, V.cpu().numpy(),
                    comp_scale=[1.0 / denom], snp_weight=w)
    args = (st._true_widths_dev, st._means_by_call, st._inv_by_call, torch.as_tensor(wb), denom)
    kw = dict(n=st.n, n_calls=st._n_calls)
    a = kv_impl.kv_impl_snp_weighted_streamed(V, *args, pop_block=st._pop_cached, **kw)
    blocks = [st._pop_cached(c) for c in range(st._n_calls)]
    b = kv_impl.kv_impl_snp_weighted_streamed(V, *args, pop_block=lambda c: blocks[c], **kw)
    c = st.snp_weighted_kv(V, w, denom)
    for out in (a, b, c):
        assert tuple(out.shape) == (st.n, 5)
        assert rel(out.cpu(), ref) < TOL
    v1 = kv_impl.kv_impl_snp_weighted_streamed(V[:, 2], *args, pop_block=st._pop_cached, **kw)
    assert v1.shape == (st.n,)
    assert rel(v1.cpu()[:, None], ref[:, 2:3]) < TOL
    # Unit weights and denom = m_eff give the plain normalised operator.
    ones = st.snp_weighted_kv(V, np.ones(st.m, np.float32), float(st._eff_m_const))
    assert rel(ones.cpu(), og.kv_f64(codes, st._means_host, st._inv_sds_host, V.cpu().numpy(),
                                     comp_scale=[1 / float(st._eff_m_const)])) < TOL
