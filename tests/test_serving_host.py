"""Host logic of the serving batcher on CPU (no device work).

The batcher's launch is replaced by a fake that maps every column through
the same column-wise function (out = 3 V + column-independent offset), so
an application must come back equal to that function however its columns
were split across launches.  Covered: launches fill to the column limit,
an application wider than the rest of a launch continues in the next one,
every application completes exactly once, a failing launch fails exactly the
applications it carried, and an empty block returns at once.  The server's
admission rule (active limit, statistics slots for subset requests, HBM
budget) and its request validation are checked on a server object built
without its device set-up."""
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
    b.launch_ms = {}
    b.launch_events = []
    b._events_base = 0
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


def _bare_server(n=100, max_active=2, budget=1e6):
    """A REMLServer without its device set-up or admission thread."""
    srv = serving.REMLServer.__new__(serving.REMLServer)
    srv.st = types.SimpleNamespace(n=n, dev=torch.device("cpu"))
    srv.max_active = max_active
    srv.budget = float(budget)
    srv._free_slots = serving.deque(range(1, max_active + 1))
    srv._active = 0
    srv._bytes_active = 0.0
    srv._closed = False
    srv._cv = threading.Condition()
    srv._waiting = serving.deque()
    srv._next_id = 0
    srv.fit_kwargs = dict(n_rand_vec=30, slq_samples=30, slq_m=30)
    return srv


def test_admission_respects_slots_budget_and_active_limit():
    srv = _bare_server(max_active=2, budget=1000.0)
    full = types.SimpleNamespace(mask=None, bytes_estimate=600.0)
    subset = types.SimpleNamespace(mask=np.ones(3, bool), bytes_estimate=600.0)
    assert srv._can_admit(full)
    srv._active, srv._bytes_active = 1, 600.0
    assert not srv._can_admit(full)             # over the HBM budget
    srv._bytes_active = 300.0
    assert srv._can_admit(full)
    srv._active = 0
    srv._bytes_active = 0.0
    assert srv._can_admit(types.SimpleNamespace(mask=None, bytes_estimate=5000.0))  # alone: always
    srv._free_slots.clear()
    assert not srv._can_admit(subset)           # no statistics slot for a subset request
    assert srv._can_admit(full)
    srv._active = 2
    assert not srv._can_admit(full)             # max_active


def test_submit_validates_and_estimates_solver_memory():
    srv = _bare_server(n=100)
    fut = srv.submit(np.zeros(100), np.ones((100, 3)))
    req = srv._waiting[-1]
    assert req.n_sub == 100 and req.covar.shape == (100, 3) and not fut.done()
    width = 3 + 1 + 30 + 30
    assert req.bytes_estimate == 4 * 100 * (8 * width + 30 * 30)
    mask = np.zeros(100, bool)
    mask[:40] = True
    srv.submit(np.zeros(40), None, mask, n_rand_vec=10)
    req = srv._waiting[-1]
    assert req.n_sub == 40 and req.fit_kwargs["n_rand_vec"] == 10
    assert [r.rid for r in srv._waiting] == [0, 1]
    with pytest.raises(ValueError, match="entries, the matrix has"):
        srv.submit(np.zeros(40), None, np.ones(99, bool))
    with pytest.raises(ValueError, match="selects no samples"):
        srv.submit(np.zeros(0), None, np.zeros(100, bool))
    with pytest.raises(ValueError, match="phenotype has 41"):
        srv.submit(np.zeros(41), None, mask)
    with pytest.raises(ValueError, match="one row per selected sample"):
        srv.submit(np.zeros(40), np.ones((39, 2)), mask)
    srv._closed = True
    with pytest.raises(RuntimeError, match="closed"):
        srv.submit(np.zeros(100))


def test_batcher_cuts_pending_columns_by_measured_launch_times():
    """With measured launch times per width the batcher opens the cheapest
    cut of the pending columns; without them it fills max_cols."""
    from coherit_gb300 import serving

    b = serving._Batcher.__new__(serving._Batcher)
    b.max_cols = 80
    b.launch_ms = {}
    assert b._first_width(96) == 80
    b.launch_ms = {16: 25.1, 32: 26.2, 48: 29.9, 64: 47.2, 80: 47.9}
    assert b._first_width(6) == 16
    assert b._first_width(48) == 48
    assert b._first_width(50) == 64          # one 64-column launch beats 48 + 16
    assert b._first_width(96) == 48          # 48 + 48 beats 80 + 16
    assert b._first_width(160) == 80


def test_projected_core_of_a_request_on_host_tensors():
    """REMLServer._projected_core (reml_model.py:863-960 for one GRM):
    Nystrom basis of the request's kernel, core diag(e) - atom I, identity
    diagonal with the request's atom; full-cohort requests share one."""
    srv = serving.REMLServer.__new__(serving.REMLServer)
    srv.st = types.SimpleNamespace(dev=torch.device("cpu"))
    srv.precond_rank = 4
    srv._full_precond = None
    srv._full_precond_lock = threading.Lock()
    g = torch.Generator().manual_seed(1)
    A = torch.randn(60, 8, generator=g)
    K = (A @ A.T / 8).float()
    srv._full_K = lambda V: K @ V
    req = types.SimpleNamespace(n_sub=60, atom=1.25, fit_kwargs={"seed": 3}, mask=None)
    conf = srv._precond_for(req, None)
    assert conf is srv._precond_for(req, None)            # shared by full-cohort requests
    U = conf.U.double()
    assert conf.total_rank == 4 and conf.n_grm == 1 and conf.diag_mode == "scalar_identity"
    torch.testing.assert_close(U.T @ U, torch.eye(4, dtype=torch.float64), atol=1e-4, rtol=0)
    core = conf.core_atoms[0].double()
    ev = torch.diagonal(core) + 1.25
    torch.testing.assert_close(core - torch.diag(torch.diagonal(core)),
                               torch.zeros(4, 4, dtype=torch.float64))
    # The basis spans the leading eigenvectors: U^T K U = diag(e).
    torch.testing.assert_close((U.T @ K.double() @ U).diagonal(), ev, atol=1e-3, rtol=1e-3)
    assert float(conf.diag_atoms[0]) == 1.25
    sub = types.SimpleNamespace(n_sub=60, atom=0.5, fit_kwargs={}, mask=np.ones(60, bool))
    other = srv._precond_for(sub, lambda V: K @ V)       # a subset request builds its own
    assert other is not conf
    srv.precond_rank = 0
    assert srv._precond_for(req, None) is None
