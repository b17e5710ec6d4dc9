"""Host-side helpers of bench.py (no GPU): the event-list comparison behind the bench line's
`event_lists` figures."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from redgb import types as T  # noqa: E402


def test_event_list_comparison():
    import bench
    a = [(0, 1, 5, 6, 10.0), (0, 1, 5, 6, 20.0), (1, 2, 3, 4, 5.0), (2, 3, 7, 8, 40.0)]
    b = [(0, 1, 5, 6, 10.0), (1, 2, 3, 4, 5.0), (2, 3, 7, 9, 30.0)]
    out = bench._compare_events(a, b, 4)
    assert not out["identical"]
    assert out["n"] == 4 and out["n_fp64"] == 3
    assert out["only_here"] == 2 and out["only_fp64"] == 1
    assert out["disks_identical"] == 2  # disks 0 and 2 differ; 1 and 3 agree
    assert out["first_difference_yr"] == 20.0 / T.YEAR  # the second (0, 1, 5, 6) record
    same = bench._compare_events(a, list(a), 4)
    assert same["identical"] and same["first_difference_yr"] is None and same["disks_identical"] == 4
