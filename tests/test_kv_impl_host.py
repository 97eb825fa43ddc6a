"""Host side of the dense kv_impl shims on CPU: the per-call effect rows of
the prediction entry points (kv_impl.py:524-724) laid out as the columns of
one Z B launch, and their argument checks (raised before any device call)."""
import types

import numpy as np
import pytest
import torch

from coherit_gb300 import kv_impl


def _ref_stack(bs, tw, calls=None):
    C, n_calls, _ = bs.shape
    parts = []
    for c in range(n_calls):
        keep = calls is None or c in calls
        parts.append(bs[:, c, : tw[c]].T if keep else np.zeros((tw[c], C)))
    return np.concatenate(parts)


@pytest.mark.parametrize("calls", [None, [2, 0], [1]])
def test_b_rows_stack_into_cache_order(calls):
    rng = np.random.default_rng(0)
    tw = np.array([5, 8, 3])
    bs = rng.normal(size=(4, 3, 8)).astype(np.float32)
    bs[:, 0, 5:] = 99.0          # beyond a call's true width: ignored
    bs[:, 2, 3:] = 99.0
    B = kv_impl._stack_b_by_call(torch.as_tensor(bs), torch.as_tensor(tw), calls)
    assert B.dtype == torch.float32 and tuple(B.shape) == (16, 4)
    np.testing.assert_array_equal(B.numpy(), _ref_stack(bs, tw, calls))


def test_same_stream_multi_argument_checks():
    f = kv_impl.zxb_impl_same_stream_multi
    args = dict(true_widths=[4], means_by_call=None, inv_by_call=None, n=3, pop_block=None)
    with pytest.raises(ValueError, match="n_components, n_calls"):
        f(np.zeros((2, 4)), n_calls=1, **args)
    with pytest.raises(ValueError, match="at least one component"):
        f(np.zeros((0, 1, 4)), n_calls=1, **args)
    with pytest.raises(ValueError, match="call mismatch: expected 2, got 1"):
        f(np.zeros((2, 1, 4)), n_calls=2, **args)
    with pytest.raises(ValueError, match="code 3"):
        f(np.zeros((2, 1, 4)), n_calls=1, missing_val=-127, **args)


def test_multi_streamed_argument_checks():
    f = kv_impl.zxb_impl_multi_streamed
    st = types.SimpleNamespace(_n_calls=2)
    with pytest.raises(ValueError, match="length mismatch: expected 1, got 2"):
        f([np.zeros((2, 4)), np.zeros((2, 4))], [st], [])
    with pytest.raises(ValueError, match="at least one streamer"):
        f([], [], [])
    with pytest.raises(ValueError, match=r"b_by_call_list\[0\] to be 2D"):
        f([np.zeros(4)], [st], [])
    with pytest.raises(ValueError, match="expected n_calls=2, got 3"):
        f([np.zeros((3, 4))], [st], [])


def test_zxb_streamed_shape_checks():
    """kv_impl.py:538-571 of the reference."""
    f = kv_impl.zxb_impl_streamed
    b = np.zeros((2, 8), np.float32)
    ok = dict(true_widths=np.array([8, 8]), means_by_call=np.zeros((2, 8)),
              inv_by_call=np.zeros((2, 8)))
    for bad, match in ((dict(true_widths=np.array([8])), "true_widths must have shape"),
                       (dict(means_by_call=np.zeros(8)), "means_by_call must have shape"),
                       (dict(inv_by_call=np.zeros((2, 7))), "inv_by_call shape mismatch")):
        args = {**ok, **bad}
        with pytest.raises(ValueError, match=match):
            f(b, args["true_widths"], args["means_by_call"], args["inv_by_call"], n=3, n_calls=2,
              pop_block=None)


@pytest.mark.parametrize("shape", [(5,), (5, 3)])
def test_no_call_blocks_give_zero(shape):
    """n_calls == 0: the accumulator is returned untouched (kv_impl.py:308-309,
    :358-359 of the reference), without any device work."""
    V = torch.ones(shape)
    z = np.zeros((0, 4), np.float32)
    out = kv_impl.kv_impl_streamed(V, np.zeros(0, np.int32), z, z, 1.0, n=5, n_calls=0,
                                   pop_block=None)
    assert tuple(out.shape) == shape and float(out.abs().sum()) == 0.0
    out = kv_impl.kv_impl_snp_weighted_streamed(V, np.zeros(0, np.int32), z, z, z, 2.0, n=5,
                                                n_calls=0, pop_block=None)
    assert tuple(out.shape) == shape and float(out.abs().sum()) == 0.0
    with pytest.raises(ValueError, match="code 3"):
        kv_impl.kv_impl_snp_weighted_streamed(V, np.zeros(0, np.int32), z, z, z, 2.0, n=5,
                                              n_calls=0, pop_block=None, missing_val=-127)
