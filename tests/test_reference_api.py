"""The package's call surface against the reference's (tests/golden/reference_api.json).

Every public function and method of the replaced reference modules exists
here and accepts the reference's parameters: the reference's positional
parameters are a prefix of ours, and each of its keyword-only parameters is
accepted by name.  FitConfig has the reference's fields and defaults (the
device-path additions aside), FitResult its fields, and the export table
every reference name of these layers.  The fixture is written from the
reference's sources by tests/golden/make_reference_api.py.
"""
import ast
import importlib
import inspect
import json
import os

import pytest

from coherit_gb300 import reml_model

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "reference_api.json")
API = json.load(open(GOLDEN))

# FitConfig defaults this package changes on purpose, with the reason.
FITCONFIG_DEFAULTS_CHANGED = {}
# Exports of the reference outside the operator/solver/model/SMILE/GWAS layers.
EXPORTS_OUT_OF_SCOPE = {
    "GenoBlockSource", "BedGenoSource", "PgenGenoSource",          # host readers (I/O layer)
    "CovariateTransform", "load_pheno_covar_aligned",             # phenotype/covariate I/O
    "load_pheno_covar_aligned_with_transform", "load_covar_aligned",
    "suggest_call_width", "PlanResult",                           # resource planner
    "LassoPathConfig", "fit_weighted_lasso_with_covariates",      # LASSO coordinate descent
    "AdmixtureQ", "load_admixture_q_aligned",                     # admixture covariance
}


def _resolve(module, dotted):
    obj = module
    for part in dotted.split("."):
        obj = inspect.getattr_static(obj, part)
    if isinstance(obj, (staticmethod, classmethod)):
        obj = obj.__func__
    return obj


ENTRIES = [(m, name) for m, entries in sorted(API["modules"].items()) for name in sorted(entries)]


@pytest.mark.parametrize("module,name", ENTRIES, ids=[f"{m}.{n}" for m, n in ENTRIES])
def test_entry_accepts_reference_parameters(module, name):
    ref = API["modules"][module][name]
    obj = _resolve(importlib.import_module(f"coherit_gb300.{module}"), name)
    if isinstance(obj, property):
        return                                           # attribute access, no parameters
    params = inspect.signature(obj).parameters
    kinds = inspect.Parameter
    positional = [p for p, v in params.items()
                  if v.kind in (kinds.POSITIONAL_ONLY, kinds.POSITIONAL_OR_KEYWORD)]
    assert positional[:len(ref["positional"])] == ref["positional"], (positional, ref)
    has_var_kw = any(v.kind == kinds.VAR_KEYWORD for v in params.values())
    by_name = {p for p, v in params.items() if v.kind != kinds.POSITIONAL_ONLY}
    for kw in ref["keyword_only"]:
        assert kw in by_name or has_var_kw, (kw, list(params))


def test_fitconfig_fields_and_defaults():
    ours = {f.name: f for f in reml_model.FitConfig.__dataclass_fields__.values()}
    for name, default in API["FitConfig"].items():
        assert name in ours, name
        if default is None or name in FITCONFIG_DEFAULTS_CHANGED:
            continue
        value = ours[name].default
        assert value == ast.literal_eval(default), (name, value, default)


def test_fitresult_fields():
    ours = set(reml_model.FitResult.__dataclass_fields__)
    assert set(API["FitResult"]) <= ours


def test_exports_cover_the_reference_layers():
    import coherit_gb300

    missing = set(API["exports"]) - set(coherit_gb300.__all__) - EXPORTS_OUT_OF_SCOPE
    assert not missing, sorted(missing)
