"""Host-side pieces of the bench line (no GPU): strict JSON for non-finite
values and the time-to-RMSE comparisons."""
import json
import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_non_finite_values_become_null():
    line = {"a": float("nan"), "b": [1.0, float("inf"), (2, float("-inf"))], "c": {"d": 3.5, "e": "x"}}
    out = json.loads(json.dumps(bench.finite(line), allow_nan=False))
    assert out == {"a": None, "b": [1.0, None, [2, None]], "c": {"d": 3.5, "e": "x"}}


def _traj(rmses, ms_per_epoch):
    return [(e + 1, (e + 1) * ms_per_epoch, r, None) for e, r in enumerate(rmses)]


def test_time_to_rmse_targets_the_plain_final():
    tuned = _traj([0.5, 0.3, 0.2, 0.105], 1.0)
    plain = _traj([0.5, 0.35, 0.2, 0.1], 4.0)
    r = bench._ttr(tuned, plain)
    assert math.isclose(r["target"], 0.101)
    # the tuned path ends 5 % above plain's final: it never reaches 1.01 x of it
    assert r["tuned_ms"] is None and r["speedup"] is None
    assert r["plain_epochs"] == 4 and r["plain_ms"] == 16.0
    # at 1.01 x the worse final both reach the level; the ratio is of device times
    c = r["at_common_level"]
    assert math.isclose(c["target"], 0.105 * 1.01)
    assert c["tuned_epochs"] == 4 and c["plain_epochs"] == 4
    assert math.isclose(c["speedup"], 16.0 / 4.0)


def test_time_to_rmse_when_the_tuned_path_is_better():
    tuned = _traj([0.5, 0.2, 0.09, 0.08], 1.0)
    plain = _traj([0.5, 0.3, 0.12, 0.1], 3.0)
    r = bench._ttr(tuned, plain)
    assert r["tuned_epochs"] == 3 and math.isclose(r["tuned_ms"], 3.0)
    assert r["plain_epochs"] == 4 and math.isclose(r["speedup"], 12.0 / 3.0)
    # the worse final is plain's, so both comparisons coincide
    assert r["at_common_level"]["speedup"] == r["speedup"]
