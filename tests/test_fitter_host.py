"""Fitter assembly on CPU with stand-in streamers (no device work): source
precedence, dense-before-sparse ordering and the reference's error
messages (reml_model.py:448-666)."""
import pytest

from coherit_gb300 import reml_model
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter


class _Dense:
    has_sparse_backend = False

    def __init__(self, source=None, *, bed_prefix=None, **kw):
        self.source, self.bed_prefix, self.n = source, bed_prefix, 10


class _Rare(_Dense):
    has_sparse_backend = True


@pytest.fixture
def fakes(monkeypatch):
    import coherit_gb300.sparse_stream as ss

    monkeypatch.setattr(reml_model, "GenoBlockStreamer", _Dense)
    monkeypatch.setattr(ss, "SparseGenoBlockStreamer", _Rare)


def test_sources_take_precedence_over_bed_prefix(fakes):
    f = InfinitesimalREMLFitter(FitConfig(sources=["s1", "s2"], bed_prefix="ignored"))
    assert [s.source for s in f.streamers] == ["s1", "s2"]
    assert all(s.bed_prefix is None for s in f.streamers)
    assert not f._has_sparse and f._n_dense_streamers == 2


def test_bed_prefixes_and_rare_streamers_follow_dense(fakes):
    f = InfinitesimalREMLFitter(FitConfig(bed_prefix=["a", "b"], rare_bed_prefix="r",
                                          rare_sources=["rs"]))
    assert [type(s).__name__ for s in f.streamers] == ["_Dense", "_Dense", "_Rare", "_Rare"]
    assert f._has_sparse and f._n_dense_streamers == 2
    assert f._sparse_streamers == tuple(f.streamers[2:])


def test_no_source_and_ordering_errors(fakes):
    with pytest.raises(ValueError, match="At least one dense or sparse"):
        InfinitesimalREMLFitter(FitConfig())
    with pytest.raises(ValueError, match="must follow the dense"):
        InfinitesimalREMLFitter(FitConfig(), streamers=[_Rare(), _Dense()])


def test_smile_rejects_rare_variant_streamers(fakes):
    with pytest.raises(ValueError, match="dense-only fits"):
        InfinitesimalREMLFitter(FitConfig(bed_prefix="a", rare_bed_prefix="r",
                                          smile_identity=True))


class _Operator:
    """Single-GRM streamer stand-in with the attributes the set-up cache keys on."""

    has_sparse_backend = False
    n_components = 1

    def __init__(self):
        import numpy as np
        import torch

        self.n, self.m = 8, 16
        self.dev = torch.device("cpu")
        self._means_by_call = np.zeros(16)
        self.closed = 0

    def kv(self, V, precision=None):
        return V

    def diag(self):
        import torch

        return torch.ones(self.n)

    def weighted_component_hv(self, tg, te, V, precision=None):
        return V

    def close(self):
        self.closed += 1


def _recording_fit(monkeypatch):
    import numpy as np

    captured = []

    def fit(**kwargs):
        captured.append((kwargs["K_mvs"], kwargs["probe_cache"]))
        diag = {"genetic_trace_atoms": np.ones(1), "residual_trace_atoms": np.ones(1),
                "loglik": 0.0}
        return np.array([0.3, 0.7]), [], diag

    monkeypatch.setattr(reml_model, "fit_reml", fit)
    return captured


# tests/test_reml_probe_cache.py:16-52 of the reference
def test_cached_setup_is_reused_and_invalidated_by_new_statistics(monkeypatch):
    import numpy as np

    captured = _recording_fit(monkeypatch)
    st = _Operator()
    fitter = InfinitesimalREMLFitter(FitConfig(cache_reml_setup=True, precond_rank=0), [st])
    try:
        fitter.fit_infinitesimal(np.ones(8))
        fitter.fit_infinitesimal(np.arange(8.0))
        assert captured[0][0] is captured[1][0]
        assert captured[0][1] is captured[1][1]
        st._means_by_call = np.ones(16)          # a new standardisation
        fitter.fit_infinitesimal(np.arange(8.0))
        assert captured[2][0] is not captured[1][0]
        assert captured[2][1] is not captured[1][1]
    finally:
        fitter.close()
    assert fitter._reml_fit_setup is None
    assert fitter._reml_probe_cache.kvrand_stack is None
    assert st.closed == 1 and fitter.streamers == []
    with pytest.raises(RuntimeError, match="closed"):
        fitter.fit_infinitesimal(np.ones(8))


def test_uncached_setup_is_rebuilt_and_shares_no_probe_cache(monkeypatch):
    import numpy as np

    captured = _recording_fit(monkeypatch)
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=0), [_Operator()])
    fitter.fit_infinitesimal(np.ones(8))
    fitter.fit_infinitesimal(np.ones(8))
    assert captured[0][0] is not captured[1][0]
    assert captured[0][1] is None and captured[1][1] is None


def test_close_tolerates_streamers_that_fail_to_close():
    class _Failing(_Operator):
        def close(self):
            raise RuntimeError("already closed")

    good = _Operator()
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=0), [_Failing(), good])
    fitter.close()
    assert good.closed == 1 and fitter.streamers == []
