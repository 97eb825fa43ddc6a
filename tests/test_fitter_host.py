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
