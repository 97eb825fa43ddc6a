"""Host logic of the serving batcher on CPU (no device work).

The batcher's launch is replaced by a fake that maps every column through
the same column-wise function (out = 3 V + column-independent offset), so
an application must come back equal to that function however its columns
were split across launches.  Covered: launches fill to the column limit,
an application wider than the rest of a launch continues in the next one,
every application completes exactly once, a failing launch fails exactly the
applications it carried, and an empty block returns at once."""
import threading
import types

import numpy as np
import pytest
import torch

from coherit_gb300 import serving


def _fake_batcher(max_cols, fail_when=None):
    b = serving._Batcher.__new__(serving._Batcher)
    b.st = types.SimpleNamespace(op_stats={"apps": 0, "cols": 0})
    b.prec = 0
    b.window_s = 0.05
    b.max_cols = int(max_cols)
    b.lib_lock = threading.Lock()
    b.cv = threading.Condition()
    b.pending = []
    b.n_active = 0
    b.stop = False
    b.launches = 0
    b.columns = 0
    b.requests_per_launch = []
    b.last_launch = None
    b._busy_cap_s = 0.25
    b.widths = []

    def launch(self, pieces):
        K = sum(hi - lo for _, lo, hi in pieces)
        assert 0 < K <= self.max_cols
        if fail_when is not None and fail_when(pieces):
            raise RuntimeError("launch failed")
        self.widths.append(K)
        self.launches += 1
        self.columns += K
        self.requests_per_launch.append(len({id(op) for op, _, _ in pieces}))
        for op, lo, hi in pieces:
            op.out[:, lo:hi] = 3.0 * op.V[:, lo:hi] + 1.0

    b._launch = types.MethodType(launch, b)
    b.thread = threading.Thread(target=b._loop, daemon=True)
    b.thread.start()
    return b


def _req(n):
    return types.SimpleNamespace(n_sub=n, idx=None, slot=0)


def _run_concurrently(b, blocks):
    """Submit every block from its own thread (as fits do); collect results."""
    b.set_active(len(blocks))
    out, errs = [None] * len(blocks), [None] * len(blocks)

    def worker(i, V):
        try:
            out[i] = b.apply(_req(V.shape[0]), V, 1.0, None)
        except Exception as e:  # noqa: BLE001 - recorded for the test
            errs[i] = e
        finally:
            b.set_active(-1)

    ts = [threading.Thread(target=worker, args=(i, V)) for i, V in enumerate(blocks)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=30)
    return out, errs


def test_applications_split_across_launches_come_back_whole():
    rng = np.random.default_rng(0)
    widths = [50, 50, 10, 79, 1, 33]
    blocks = [torch.as_tensor(rng.normal(size=(12, w)).astype(np.float32)) for w in widths]
    b = _fake_batcher(max_cols=80)
    try:
        out, errs = _run_concurrently(b, blocks)
    finally:
        b.close()
    assert errs == [None] * len(blocks)
    for V, o in zip(blocks, out):
        torch.testing.assert_close(o, 3.0 * V + 1.0)
    assert b.columns == sum(widths)
    assert all(w <= 80 for w in b.widths)


def test_vector_and_empty_blocks():
    b = _fake_batcher(max_cols=16)
    try:
        b.set_active(1)
        v = torch.arange(5, dtype=torch.float32)
        torch.testing.assert_close(b.apply(_req(5), v, 1.0, None), 3.0 * v + 1.0)
        empty = b.apply(_req(5), torch.zeros((5, 0)), 1.0, None)
        assert tuple(empty.shape) == (5, 0)
    finally:
        b.close()
    assert b.launches == 1


def test_a_failing_launch_fails_the_applications_it_carried():
    rng = np.random.default_rng(1)
    blocks = [torch.as_tensor(rng.normal(size=(4, w)).astype(np.float32)) for w in (8, 8, 8)]
    marker = blocks[1]

    def fail_when(pieces):
        return any(op.V.data_ptr() == marker.data_ptr() for op, _, _ in pieces)

    b = _fake_batcher(max_cols=8, fail_when=fail_when)
    try:
        out, errs = _run_concurrently(b, blocks)
    finally:
        b.close()
    assert isinstance(errs[1], RuntimeError)
    for i in (0, 2):
        assert errs[i] is None
        torch.testing.assert_close(out[i], 3.0 * blocks[i] + 1.0)


def test_closed_batcher_rejects_new_work():
    b = _fake_batcher(max_cols=8)
    b.close()
    with pytest.raises(RuntimeError, match="closed"):
        b.apply(_req(3), torch.ones((3, 2)), 1.0, None)


def test_split_application_whose_first_launch_fails_does_not_hang():
    V = torch.ones((4, 12))
    calls = []

    def fail_when(pieces):
        calls.append([(lo, hi) for _, lo, hi in pieces])
        return len(calls) == 1  # the launch holding columns 0..8 fails

    b = _fake_batcher(max_cols=8, fail_when=fail_when)
    try:
        out, errs = _run_concurrently(b, [V])
    finally:
        b.close()
    assert isinstance(errs[0], RuntimeError)
    assert calls[0] == [(0, 8)]
    assert b.pending == []
