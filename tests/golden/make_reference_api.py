"""Write reference_api.json: the public call surface of the reference modules
this package replaces, read from their sources with ast (no import).

Run from the repository root, giving the reference checkout as the argument
or in COHERIT_REFERENCE_ROOT:

    python tests/golden/make_reference_api.py <reference checkout>

Recorded per module: the parameter names of every public top-level function
and of every public method (and __init__) of every public class, split into
positional and keyword-only; the fields and defaults of FitConfig and
FitResult; the package export table.  tests/test_reference_api.py checks the
package against this file.
"""
from __future__ import annotations

import ast
import json
import os
import sys

MODULES = ["reml", "slq", "precond", "pcg", "kv_impl", "smile_block_w", "reml_model", "gwas",
           "geno_stream", "sparse_stream", "block_backend"]


def _params(fn: ast.FunctionDef) -> dict:
    a = fn.args
    return {"positional": [x.arg for x in a.posonlyargs + a.args],
            "keyword_only": [x.arg for x in a.kwonlyargs]}


def _public(name: str) -> bool:
    return not name.startswith("_") or name == "__init__"


def surface(path: str) -> dict:
    tree = ast.parse(open(path, encoding="utf-8").read())
    out = {}
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and _public(node.name):
            out[node.name] = _params(node)
        elif isinstance(node, ast.ClassDef) and not node.name.startswith("_"):
            for item in node.body:
                if isinstance(item, ast.FunctionDef) and _public(item.name):
                    out[f"{node.name}.{item.name}"] = _params(item)
    return out


def dataclass_fields(path: str, cls: str) -> dict:
    tree = ast.parse(open(path, encoding="utf-8").read())
    for node in tree.body:
        if isinstance(node, ast.ClassDef) and node.name == cls:
            return {s.target.id: (None if s.value is None else ast.unparse(s.value))
                    for s in node.body if isinstance(s, ast.AnnAssign)}
    raise KeyError(cls)


def exports(path: str) -> dict:
    tree = ast.parse(open(path, encoding="utf-8").read())
    for node in tree.body:
        if isinstance(node, ast.AnnAssign) and getattr(node.target, "id", "") == "_EXPORTS":
            return ast.literal_eval(node.value)
    raise KeyError("_EXPORTS")


def main(root: str) -> None:
    api = {"modules": {m: surface(os.path.join(root, f"{m}.py")) for m in MODULES},
           "FitConfig": dataclass_fields(os.path.join(root, "reml_model.py"), "FitConfig"),
           "FitResult": dataclass_fields(os.path.join(root, "reml_model.py"), "FitResult"),
           "exports": exports(os.path.join(root, "__init__.py"))}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_api.json"), "w") as f:
        json.dump(api, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("COHERIT_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_reference_api.py <reference checkout> "
                 "(or set COHERIT_REFERENCE_ROOT)")
    main(root)
