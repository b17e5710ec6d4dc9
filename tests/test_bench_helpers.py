"""Host-side helpers of bench.py (no GPU): the event-list comparison behind the bench line's
`event_lists` figures, and the margin of a record to its event's threshold."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from redgb import types as T  # noqa: E402


def test_event_list_comparison():
    import bench
    a = [(0, 1, 5, 6, 10.0, 0.1), (0, 1, 5, 6, 20.0, -0.002), (1, 2, 3, 4, 5.0, 0.0), (2, 3, 7, 8, 40.0, -1e-6)]
    b = [(0, 1, 5, 6, 10.0, 0.1), (1, 2, 3, 4, 5.0, 0.0), (2, 3, 7, 9, 30.0, -0.5)]
    out = bench._compare_events(a, b, 4)
    assert not out["identical"]
    assert out["n"] == 4 and out["n_fp64"] == 3
    assert out["only_here"] == 2 and out["only_fp64"] == 1
    assert out["disks_identical"] == 2  # disks 0 and 2 differ; 1 and 3 agree
    assert out["first_difference_yr"] == 20.0 / T.YEAR  # the second (0, 1, 5, 6) record
    recs = out["differing_records"]
    assert [(r["list"], r["disk"], r["id2"]) for r in recs] == [("here", 0, 6), ("fp64", 2, 9), ("here", 2, 8)]
    assert [r["margin"] for r in recs] == [-0.002, -0.5, -1e-6]
    assert out["largest_abs_margin"] == 0.5
    same = bench._compare_events(a, list(a), 4)
    assert same["identical"] and same["first_difference_yr"] is None and same["disks_identical"] == 4
    assert same["differing_records"] == [] and same["largest_abs_margin"] is None


def test_event_margins():
    """Each record's distance to its threshold: radius sum for collisions, mutual Hill radius
    (star distances from the barycentre) for close encounters, the two radii for ejection and
    hit-star."""
    import bench
    rec = np.zeros(1, T.EVENT)[0]
    rec["event_name"] = T.EVENT_COLLISION
    rec["d"] = 0.9e-4
    rec["p1"]["radius"], rec["p2"]["radius"] = 0.6e-4, 0.4e-4
    assert abs(bench.event_margin(rec) - (-0.1)) < 1e-12
    rec["event_name"] = T.EVENT_CLOSE_ENCOUNTER
    rec["p1"]["mass"], rec["p2"]["mass"] = 9.55e-4, 1e-9
    rec["r1"]["x"], rec["r2"]["x"] = 5.0, 4.0
    rh = ((9.55e-4 + 1e-9) / 3.0) ** (1.0 / 3.0) * 4.5
    rec["d"] = 3.0 * rh * 1.25
    assert abs(bench.event_margin(rec) - 0.25) < 1e-12
    rec["event_name"] = T.EVENT_EJECTION
    rec["d"] = 101.0
    assert abs(bench.event_margin(rec) - 0.01) < 1e-12
    rec["event_name"] = T.EVENT_HIT_CENTRUM
    rec["d"] = 0.04
    assert abs(bench.event_margin(rec) - (-0.2)) < 1e-12
