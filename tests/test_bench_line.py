"""The bench line is strict JSON: phases a run skips (the FP64 and accuracy
phases of a profiling run) are printed as null, not NaN."""
import json
import math

import bench


def _strict(s):
    def bad(c):
        raise ValueError("non-finite constant " + c)
    return json.loads(s, parse_constant=bad)


def test_skipped_phases_print_as_null():
    line = {"value": 230.7, "accuracy": {"rel_err_E_per_atom": float("nan"), "steps": 20},
            "fp64": {"value": float("nan")}, "list": [1.0, float("inf")], "name": "x"}
    out = _strict(json.dumps(bench.finite_or_null(line)))
    assert out["accuracy"]["rel_err_E_per_atom"] is None and out["accuracy"]["steps"] == 20
    assert out["fp64"]["value"] is None and out["list"] == [1.0, None] and out["value"] == 230.7
    assert not any(isinstance(v, float) and math.isnan(v) for v in out["accuracy"].values())
