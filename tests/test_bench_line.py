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


def test_reference_arm_line_on_a_small_grid():
    """bench.py --impl reference (the FP64 CPU path on the host cores) prints
    one strict-JSON line with the contract's keys; --grid names the grid it ran."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--grid", "32",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=300, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = _strict(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "steps", "warmup", "ms_per_step", "higher_is_better", "dtype",
              "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "steps/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert "32^3" in line["config"]["workload"] and line["config"]["grid"] == [32, 32, 32]
