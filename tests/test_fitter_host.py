"""The fitter's host logic on CPU with stand-in streamers and a recorded
fit_reml (no device work): source precedence, dense-before-sparse ordering
and the reference's error messages (reml_model.py:448-666), config fields
reaching the streamers, the cached set-up and close() (:1818-1871), and
replicate fits with their Monte-Carlo errors (:1891-1977)."""
import pytest

from coherit_gb300 import reml_model
from coherit_gb300.reml_model import FitConfig, InfinitesimalREMLFitter


class _Dense:
    has_sparse_backend = False

    def __init__(self, source=None, *, bed_prefix=None, **kw):
        self.source, self.bed_prefix, self.n, self.kw = source, bed_prefix, 10, kw


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
                "loglik": 0.0, "ai": np.eye(2), "grad": np.zeros(2)}
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


def test_replicate_fits_report_mean_and_monte_carlo_errors(monkeypatch):
    """reml_model.py:1891-1977: seeds seed + 9973 r, mean components, Monte-Carlo SE."""
    import numpy as np

    seeds = []
    params = {0: [0.2, 0.8], 9973: [0.4, 0.6], 19946: [0.3, 0.9]}

    def fit(**kwargs):
        seeds.append(kwargs["seed"])
        diag = {"genetic_trace_atoms": np.array([2.0]), "residual_trace_atoms": np.ones(1),
                "loglik": -1.0, "ai": np.eye(2), "grad": np.zeros(2)}
        return np.array(params[kwargs["seed"]]), [{"iter": 1}], diag

    monkeypatch.setattr(reml_model, "fit_reml", fit)
    cfg = FitConfig(precond_rank=0, n_reml_reps=3, capture_reml_diagnostics=True)
    res = InfinitesimalREMLFitter(cfg, [_Operator()]).fit_infinitesimal(np.ones(8))
    assert seeds == [0, 9973, 19946]
    reps = np.array(list(params.values()))
    np.testing.assert_allclose(res.rep_var_components, reps)
    np.testing.assert_allclose(res.var_components, reps.mean(axis=0))
    se = np.sqrt(np.sum((reps - reps.mean(axis=0)) ** 2, axis=0) / 6)
    np.testing.assert_allclose(res.monte_carlo_se_var, se)
    h2 = 2 * reps[:, 0] / (2 * reps[:, 0] + reps[:, 1])
    assert res.monte_carlo_se_h2 == pytest.approx(np.sqrt(np.sum((h2 - h2.mean()) ** 2) / 6))
    mean = reps.mean(axis=0)
    assert res.heritability == pytest.approx(2 * mean[0] / (2 * mean[0] + mean[1]))
    assert res.diagnostics is None and res.final_ai is None and res.final_loglik is None


def test_single_fit_result_and_effects_flag(monkeypatch):
    import numpy as np

    _recording_fit(monkeypatch)
    calls = []
    monkeypatch.setattr(InfinitesimalREMLFitter, "estimate_effects",
                        lambda self, y, *, var_components, covar=None: calls.append(
                            (np.asarray(var_components), covar)) or "effects")
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=0), [_Operator()])
    res = fitter.fit_infinitesimal(np.ones(8))
    assert res.effects is None and res.rep_var_components is None
    assert res.monte_carlo_se_h2 is None and res.diagnostics is None
    np.testing.assert_array_equal(res.final_ai, np.eye(2))
    assert res.final_loglik == 0.0 and res.heritability == pytest.approx(0.3)
    res = fitter.fit_infinitesimal(np.ones(8), None, 0.5, None, True)
    assert res.effects == "effects"
    np.testing.assert_array_equal(calls[0][0], [0.3, 0.7])
    with pytest.raises(NotImplementedError):
        fitter.fit_infinitesimal(np.ones(8), mean_information=object())


def test_config_fields_reach_the_streamers(fakes):
    ov = [(1, 2), (3, 4)]
    f = InfinitesimalREMLFitter(FitConfig(sources=["a", "b"], standardization_overrides=ov,
                                          keep_host_stats=False, cpu_threads=3, ring_depth=2,
                                          source_build_chunk_width=64))
    assert [s.kw["standardization_override"] for s in f.streamers] == ov
    kw = f.streamers[0].kw
    assert kw["keep_host_stats"] is False and kw["build_threads"] == 3
    assert kw["ring_depth"] == 2 and kw["source_build_chunk_width"] == 64
    with pytest.raises(ValueError, match="number of dense sources"):
        InfinitesimalREMLFitter(FitConfig(sources=["a", "b"], standardization_overrides=[ov[0]]))
    with pytest.raises(ValueError, match="number of dense BED prefixes"):
        InfinitesimalREMLFitter(FitConfig(bed_prefix=["a"], standardization_overrides=ov))
    with pytest.raises(NotImplementedError, match="Admixture"):
        InfinitesimalREMLFitter(FitConfig(sources=["a"], admix_weights=[[1.0]]))


def test_config_defaults_follow_the_reference():
    cfg = FitConfig()
    assert cfg.verbose is True and cfg.n_reml_reps == 1 and cfg.keep_host_stats is True
    assert (cfg.slq_samples, cfg.slq_m, cfg.slq_mode) == (4, 8, "projected_core_residual")
    assert (cfg.precond_rank, cfg.n_rand_vec, cfg.max_pcg_iters) == (500, 100, 400)


def test_preconditioner_is_built_once_per_fitter(monkeypatch):
    """reml_model.py:1392-1407: the projected-core preconditioner is built at
    the first fit and reused by later fits of the same fitter."""
    import numpy as np

    passed = []

    def fit(**kwargs):
        passed.append(kwargs["precond_conf"])
        diag = {"genetic_trace_atoms": np.ones(1), "residual_trace_atoms": np.ones(1),
                "loglik": 0.0, "ai": np.eye(2), "grad": np.zeros(2)}
        return np.array([0.3, 0.7]), [], diag

    built = []

    def build(self, ops, var_components_init=None, theta_ref=None):
        self.precond_conf = object()
        built.append(var_components_init)
        return self.precond_conf

    monkeypatch.setattr(reml_model, "fit_reml", fit)
    monkeypatch.setattr(InfinitesimalREMLFitter, "_build_projected_core_precond", build)
    fitter = InfinitesimalREMLFitter(FitConfig(precond_rank=8), [_Operator()])
    fitter.fit_infinitesimal(np.ones(8), var_components_init=[0.5, 0.5])
    fitter.fit_infinitesimal(np.arange(8.0))
    assert len(built) == 1 and built[0] == [0.5, 0.5]
    assert passed[0] is passed[1] is fitter.precond_conf
    fitter.fit_infinitesimal(np.ones(8), precond=False)
    assert passed[2] is None
    fitter.close()
    assert fitter.precond_conf is None


def test_partition_checks_follow_the_reference(fakes):
    """reml_model.py:464-512: one dense source split into components."""
    with pytest.raises(ValueError, match="either vc_block_sizes or component_variant_indices"):
        InfinitesimalREMLFitter(FitConfig(sources=["a"], vc_block_sizes=[2],
                                          component_variant_indices=[[0, 1]]))
    with pytest.raises(ValueError, match="only for dense-only fits"):
        InfinitesimalREMLFitter(FitConfig(sources=["a"], vc_block_sizes=[2], rare_sources=["r"]))
    with pytest.raises(ValueError, match="exactly one dense source"):
        InfinitesimalREMLFitter(FitConfig(sources=["a", "b"], vc_block_sizes=[2]))
    with pytest.raises(ValueError, match="exactly one dense BED prefix"):
        InfinitesimalREMLFitter(FitConfig(bed_prefix=["a", "b"], component_variant_indices=[[0]]))
    f = InfinitesimalREMLFitter(FitConfig(sources=["a"], vc_block_sizes=[3, 7]))
    assert f.streamers[0].kw["component_block_sizes"] == [3, 7]


def test_prediction_geometry_checks():
    """reml_model.py:223-272 (without the variant-metadata files)."""
    import types

    import numpy as np

    def geo(m=10, starts=(0, 5), widths=(5, 5), part=False, cts=None, offs=(0, 10)):
        return types.SimpleNamespace(m=m, _n_calls=len(starts), _call_snp_starts=np.array(starts),
                                     _call_true_widths=np.array(widths),
                                     has_component_partition=part,
                                     _cache_to_source_variant_indices=cts,
                                     _component_snp_offsets=np.array(offs))

    check = reml_model._validate_dense_prediction_streamers
    check([geo()], [geo()])
    cases = [
        ([geo(), geo()], [geo()], "component count mismatch"),
        ([geo()], [geo(m=11)], "SNP count mismatch"),
        ([geo()], [geo(starts=(0,), widths=(10,))], "call geometry mismatch"),
        ([geo()], [geo(starts=(0, 4))], "SNP call starts mismatch"),
        ([geo()], [geo(widths=(5, 6))], "call widths mismatch"),
        ([geo(part=True)], [geo()], "partitioning mode mismatch"),
        ([geo(cts=np.arange(10))], [geo()], "variant-order mapping mismatch"),
        ([geo(cts=np.arange(10))], [geo(cts=np.arange(10)[::-1])], "source-variant order"),
        ([geo(part=True, offs=(0, 4, 10))], [geo(part=True, offs=(0, 5, 10))],
         "component block layout mismatch"),
    ]
    for train, test, match in cases:
        with pytest.raises(ValueError, match=match):
            check(train, test)
    with pytest.raises(FloatingPointError, match="Failed to stabilize GLS"):
        import torch

        reml_model._solve_small_spd(torch.tensor([[0.0, 1e3], [1e3, 0.0]]), torch.ones(2))


def test_unit_variance_components_report_no_atoms(monkeypatch):
    import numpy as np

    def fit(**kwargs):
        assert kwargs["unit_variance_components"] is True
        diag = {"loglik": -1.0, "ai": np.eye(2), "grad": np.zeros(2)}
        return np.array([0.6, 0.2]), [], diag

    monkeypatch.setattr(reml_model, "fit_reml", fit)
    cfg = FitConfig(precond_rank=0, unit_variance_components=True)
    res = InfinitesimalREMLFitter(cfg, [_Operator()]).fit_infinitesimal(np.ones(8))
    assert res.genetic_trace_atoms is None and res.residual_trace_atoms is None
    assert res.heritability == pytest.approx(0.75)


def test_reference_weights_of_the_preconditioner_kernel():
    """theta_ref (reml_model.py:808-832): the first G variance components
    clamped at zero and normalised to sum 1; uniform 1/G without them or
    when they sum to zero; too few components is an error."""
    import numpy as np

    th = reml_model._theta_ref_from_var_components
    np.testing.assert_allclose(th(3), [1 / 3] * 3)
    np.testing.assert_allclose(th(2, [0.2, 0.6, 0.5]), [0.25, 0.75], rtol=1e-6)
    np.testing.assert_allclose(th(2, [-0.1, 0.4, 0.5]), [0.0, 1.0])
    np.testing.assert_allclose(th(2, [0.0, 0.0, 1.0]), [0.5, 0.5])
    with pytest.raises(ValueError, match="length mismatch"):
        th(3, [0.1, 0.2])


def test_slq_workspace_option_reaches_fit_reml(monkeypatch):
    """FitConfig.slq_workspace_bytes replaces the reference's budget policy
    (256 MiB without gpu_budget_bytes) when set."""
    import numpy as np

    seen = []

    def fit(**kwargs):
        seen.append(kwargs["slq_workspace_bytes"])
        diag = {"genetic_trace_atoms": np.ones(1), "residual_trace_atoms": np.ones(1),
                "loglik": 0.0, "ai": np.eye(2), "grad": np.zeros(2)}
        return np.array([0.3, 0.7]), [], diag

    monkeypatch.setattr(reml_model, "fit_reml", fit)
    InfinitesimalREMLFitter(FitConfig(precond_rank=0), [_Operator()]).fit_infinitesimal(
        np.ones(8))
    InfinitesimalREMLFitter(FitConfig(precond_rank=0, slq_workspace_bytes=3 << 30),
                            [_Operator()]).fit_infinitesimal(np.ones(8))
    assert seen == [256 * 1024 ** 2, 3 << 30]
