"""The reference's output files (redgb.io) against files the reference itself wrote.

tests/golden/*_result.txt.gz, *_result.bin.gz and *_event.txt.gz are verbatim outputs of
the reference's CPU path on two seeded cases (tests/golden/make_golden.py).  Two checks:
each file parsed and written again is identical to the byte, and the same case run
through the oracle (bit-exact with the reference) and written by redgb.io reproduces the
reference's files byte for byte.
"""
import gzip
import io
import os

import numpy as np
import pytest

import helpers as H
import pyoracle
from redgb import io as rio, types as T
from redgb.driver import run_main_loop

G = H.GOLDEN


def _raw(name):
    with gzip.open(os.path.join(G, name), "rb") as f:
        return f.read()


def _case(name):
    """The case's stored initial state (exact arrays: regenerating the synthetic disk on
    another machine may round its trigonometry differently) with its body names."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(G, "make_golden.py"))
    make_golden = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(make_golden)
    names = next(d.names for n, d, _ in make_golden.cases() if n == name)
    disk, params, _, _ = H.load_fixture(name)
    disk.names = list(names)
    return disk, params


def test_text_result_round_trip():
    raw = _raw("disk_eject_hit_result.txt.gz").decode()
    rows = rio.read_result_ascii(io.StringIO(raw))
    assert len(rows) == 104
    out = io.StringIO()
    rio.write_rows_ascii(out, rows)
    assert out.getvalue() == raw


def test_binary_result_round_trip_and_agrees_with_text():
    text = rio.read_result_ascii(io.StringIO(_raw("disk_eject_hit_result.txt.gz").decode()))
    counts, last = [], None
    for row in text:
        if row.t != last:
            counts.append(0)
            last = row.t
        counts[-1] += 1
    data = _raw("disk_eject_hit_result.bin.gz")
    snaps = rio.read_result_binary(data, counts)
    out = io.BytesIO()
    rio.write_rows_binary(out, snaps)
    assert out.getvalue() == data
    flat = [row for _, rows in snaps for row in rows]
    for a, b in zip(flat, text):
        assert (a.id, a.name, a.type, a.mig_type) == (b.id, b.name, b.type, b.mig_type)
        assert H.same([a.t, a.mass, a.radius, a.density, a.cd, a.mig_stop_at, *a.r, *a.v],
                      [b.t, b.mass, b.radius, b.density, b.cd, b.mig_stop_at, *b.r, *b.v])


def test_event_lines_round_trip():
    for name in ("disk_eject_hit_event.txt.gz", "disk_si_rkf78_ce_event.txt.gz"):
        raw = _raw(name).decode()
        lines = rio.read_event_lines(io.StringIO(raw))
        assert all(len(x) == 49 for _, x in lines)
        out = io.StringIO()
        rio.write_event_lines(out, lines)
        assert out.getvalue() == raw, name


def test_writers_reproduce_reference_files_from_a_run():
    """The oracle's run of the case, written by redgb.io, is the reference's output."""
    disk, params = _case("disk_eject_hit")
    o = pyoracle.OracleSystem(disk, H.thresholds_of(params))
    H.configure(o, params)
    snaps, events, _ = run_main_loop(o, params["length_yr"] * T.YEAR, params["output_interval_yr"] * T.YEAR,
                                     radii_enhance_factor=params.get("collision_factor", 0.0) or 0.0,
                                     keep_inactive=True)
    text, binary = io.StringIO(), io.BytesIO()
    for t, r, v, p, md in snaps:
        # the reference's names: body_names[storage slot], never compacted
        rio.write_result_ascii(text, t, r, v, p, md, disk.names)
        rio.write_result_binary(binary, t, r, v, p, md, disk.names)
    assert text.getvalue() == _raw("disk_eject_hit_result.txt.gz").decode()
    assert binary.getvalue() == _raw("disk_eject_hit_result.bin.gz")
    ev = io.StringIO()
    rio.write_events(ev, events)
    assert ev.getvalue() == _raw("disk_eject_hit_event.txt.gz").decode()


def test_nan_and_negative_zero_follow_the_c_library():
    assert rio._real(float("nan")).strip() == "nan"
    assert rio._real(-float("nan")).strip() == "-nan"
    assert rio._real(-0.0).strip() == "-0.0000000000000000e+00"
    assert rio._real(1e-300).strip() == "1.0000000000000000e-300"
    assert len(rio._real(1.0)) == 25


@pytest.mark.gpu
def test_gpu_run_writes_the_reference_files(gpulib):
    """The CUDA library's run of the case, written by redgb.io: the reference's bytes."""
    from redgb import lib
    disk, params = _case("disk_eject_hit")
    s = lib.System(disk, H.thresholds_of(params))
    H.configure(s, params)
    snaps, events, _ = run_main_loop(s, params["length_yr"] * T.YEAR, params["output_interval_yr"] * T.YEAR,
                                     radii_enhance_factor=params.get("collision_factor", 0.0) or 0.0,
                                     keep_inactive=True)
    text, binary, ev = io.StringIO(), io.BytesIO(), io.StringIO()
    for t, r, v, p, md in snaps:
        rio.write_result_ascii(text, t, r, v, p, md, disk.names)
        rio.write_result_binary(binary, t, r, v, p, md, disk.names)
    rio.write_events(ev, events)
    assert text.getvalue() == _raw("disk_eject_hit_result.txt.gz").decode()
    assert binary.getvalue() == _raw("disk_eject_hit_result.bin.gz")
    assert ev.getvalue() == _raw("disk_eject_hit_event.txt.gz").decode()
