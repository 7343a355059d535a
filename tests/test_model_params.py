"""The model layer against the reference's own model files: for each golden case
(tests/golden/model_params.json, written by make_model_params.py from the reference's
dna1 / dna2 / rna2 modules), the forces of ``dnaX.forces(**same arguments)`` come in
the same order, with the same classes, default cutoffs, list buffer and, per type
pair or bond type, the same parameter values."""

import json
import math
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "model_params.json")
with open(GOLDEN) as _fh:
    CASES = json.load(_fh)


def _same(a, b, path):
    if isinstance(a, list):
        assert isinstance(b, (list, tuple)) and len(a) == len(b), path
        for k, (x, y) in enumerate(zip(a, b)):
            _same(x, y, f"{path}[{k}]")
    elif isinstance(a, bool):
        assert bool(b) == a, path
    elif isinstance(a, float):
        assert math.isclose(float(b), a, rel_tol=1e-14, abs_tol=1e-15), (path, a, b)
    else:
        assert a == b, path


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["model"] + "-" + "-".join(
    f"{k}={v}" for k, v in sorted(c["kwargs"].items())))
def test_model_parameters_match_the_reference(case):
    import importlib
    mod = importlib.import_module("oxdna.model." + case["model"])
    forces, nlist = mod.forces(**case["kwargs"])
    assert nlist.buffer == case["nlist_buffer"]
    assert [type(f).__name__ for f in forces] == [g["class"] for g in case["forces"]]
    for f, g in zip(forces, case["forces"]):
        name = g["class"]
        # the parameter declaration: the same keys, kinds and tuple widths, keyed the
        # same way, and the same keys optional
        def shape(v):
            return [shape(x) for x in v] if isinstance(v, tuple) else v.__name__
        assert {p: shape(v) for p, v in f.params._spec.items()} == g["spec"], name
        assert f.params._len_keys == g["len_keys"], name
        assert set(f.params._defaults) == set(g["defaults"]), name
        if g["default_r_cut"] is not None:
            assert math.isclose(f.default_r_cut, g["default_r_cut"], rel_tol=1e-14), name
        for key, ref in g["params"].items():
            k = tuple(key.split(",")) if "," in key else key
            ours = f.params[k]
            missing = set(ref) - set(ours)
            assert not missing, (name, key, missing)
            for p, v in ref.items():
                _same(v, ours[p], f"{case['model']} {name} {key} {p}")
            # keys the reference model leaves unset take the reference's defaults
            for p in set(ours) - set(ref):
                assert p in g["defaults"], (name, key, p)
                _same(g["defaults"][p], ours[p], f"{case['model']} {name} {key} {p} (default)")
