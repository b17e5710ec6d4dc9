"""The reference's output files: result snapshots (text and binary) and event records.

Writers produce the reference's byte layout so that its analysis tools read this
library's output unchanged; readers parse either producer's files.

* text result (pp_disk::print_result_ascii, pp_disk.cu:1685-1725): per snapshot, one line
  per active body -- id (width 8), name (30), type (2), t [day], mass, radius, density, cd,
  mig_type (2), mig_stop_at, x, y, z, vx, vy, vz [AU, AU/day]; reals in scientific
  notation with 16 digits after the point in width 25, fields separated by one space;
* binary result (pp_disk::print_result_binary, pp_disk.cu:1727-1770): per snapshot the time
  (float64), then per active body id (int32), name (NUL-terminated), type (int32), mass,
  radius, density, cd (float64), mig_type (int32), mig_stop_at, x, y, z, vx, vy, vz
  (float64), native little-endian, no padding;
* events (pp_disk::print_event_data, pp_disk.cu:1772-1848): one line per record -- name
  (width 16), t [day], d, id1, id2 (width 8), then for the survivor before, the merger
  before and the survivor after the event: mass, density, radius, position, velocity
  [AU/day] and the six orbital elements; a trailing separator ends each line.

Active bodies are those with id > 0 and a type below the padding particle (the reference
skips the others).  Real numbers follow the C library's "%.16e" (glibc: two exponent
digits at least, "nan" / "-nan", "inf" / "-inf").
"""
from __future__ import annotations

import math
import struct

import numpy as np

from . import types as T

_W_INT, _W_REAL = 8, 25
EVENT_NAMES = T.EVENT_NAMES


def _real(x, width=_W_REAL):
    x = float(x)
    if math.isnan(x):
        s = "-nan" if math.copysign(1.0, x) < 0 else "nan"
    elif math.isinf(x):
        s = "-inf" if x < 0 else "inf"
    else:
        s = "%.16e" % x
    return s.rjust(width)


def _active(md):
    return (md["id"] > 0) & (md["body_type"] < T.BODY_PADDINGPARTICLE)


def names_by_id(disk):
    """id -> name of a disk's bodies (names that follow their bodies through compactions).

    The reference itself prints body_names[i] for storage slot i and never compacts that
    list (remove_inactive_bodies, pp_disk.cu:1324-1409, moves only the records), so after a
    compaction its files name each record after the body that first held the slot.  To
    write byte-identical files, pass the disk's original name list instead, with the whole
    storage (run_main_loop(..., keep_inactive=True))."""
    return {int(disk.md[i]["id"]): disk.names[i] for i in range(disk.n_total)}


def _name(names, md, i):
    return names[int(md[i]["id"])] if isinstance(names, dict) else names[i]


# ----------------------------------------------------------------------------- results

def write_result_ascii(f, t_day, r, v, p, md, names):
    """One snapshot of the state (file units: AU, AU/day, days) as text lines; `names` is
    an id -> name map (names_by_id) or a list aligned with the records."""
    for i in np.nonzero(_active(md))[0]:
        fields = [str(int(md[i]["id"])).rjust(_W_INT), str(_name(names, md, i)).rjust(30), str(int(md[i]["body_type"])).rjust(2),
                  _real(t_day), _real(p[i]["mass"]), _real(p[i]["radius"]), _real(p[i]["density"]),
                  _real(p[i]["cd"]), str(int(md[i]["mig_type"])).rjust(2), _real(md[i]["mig_stop_at"]),
                  _real(r[i]["x"]), _real(r[i]["y"]), _real(r[i]["z"]),
                  _real(v[i]["x"]), _real(v[i]["y"]), _real(v[i]["z"])]
        f.write(" ".join(fields) + "\n")


def write_result_binary(f, t_day, r, v, p, md, names):
    """One snapshot in the reference's binary layout (f opened in binary mode)."""
    out = [struct.pack("<d", float(t_day))]
    for i in np.nonzero(_active(md))[0]:
        out.append(struct.pack("<i", int(md[i]["id"])))
        out.append(str(_name(names, md, i)).encode() + b"\0")
        out.append(struct.pack("<i", int(md[i]["body_type"])))
        out.append(struct.pack("<4d", p[i]["mass"], p[i]["radius"], p[i]["density"], p[i]["cd"]))
        out.append(struct.pack("<i", int(md[i]["mig_type"])))
        out.append(struct.pack("<7d", md[i]["mig_stop_at"], r[i]["x"], r[i]["y"], r[i]["z"],
                               v[i]["x"], v[i]["y"], v[i]["z"]))
    f.write(b"".join(out))


class ResultRow:
    __slots__ = ("id", "name", "type", "t", "mass", "radius", "density", "cd", "mig_type", "mig_stop_at", "r", "v")


def read_result_ascii(f):
    """All rows of a text result file: a list of ResultRow (names kept)."""
    rows = []
    for line in f:
        x = line.split()
        if not x:
            continue
        row = ResultRow()
        row.id, row.name, row.type = int(x[0]), x[1], int(x[2])
        row.t, row.mass, row.radius, row.density, row.cd = (float(y) for y in x[3:8])
        row.mig_type, row.mig_stop_at = int(x[8]), float(x[9])
        row.r = tuple(float(y) for y in x[10:13])
        row.v = tuple(float(y) for y in x[13:16])
        rows.append(row)
    return rows


def read_result_binary(data, counts):
    """Snapshots of a binary result file: [(t_day, [ResultRow, ...]), ...].  The layout has
    no body count, so `counts[k]` gives the number of active bodies in snapshot k."""
    out, k = [], 0
    for n in counts:
        (t,) = struct.unpack_from("<d", data, k)
        k += 8
        rows = []
        for _ in range(n):
            row = ResultRow()
            (row.id,) = struct.unpack_from("<i", data, k)
            k += 4
            end = data.index(b"\0", k)
            row.name = data[k:end].decode()
            k = end + 1
            (row.type,) = struct.unpack_from("<i", data, k)
            k += 4
            row.mass, row.radius, row.density, row.cd = struct.unpack_from("<4d", data, k)
            k += 32
            (row.mig_type,) = struct.unpack_from("<i", data, k)
            k += 4
            vals = struct.unpack_from("<7d", data, k)
            k += 56
            row.mig_stop_at, row.r, row.v = vals[0], vals[1:4], vals[4:7]
            row.t = t
            rows.append(row)
        out.append((t, rows))
    if k != len(data):
        raise ValueError(f"binary result: {len(data) - k} bytes left after {len(counts)} snapshots")
    return out


def write_rows_ascii(f, rows):
    """Text lines of parsed rows (the inverse of read_result_ascii)."""
    for row in rows:
        fields = [str(row.id).rjust(_W_INT), row.name.rjust(30), str(row.type).rjust(2), _real(row.t),
                  _real(row.mass), _real(row.radius), _real(row.density), _real(row.cd),
                  str(row.mig_type).rjust(2), _real(row.mig_stop_at)] + [_real(x) for x in row.r] + \
                 [_real(x) for x in row.v]
        f.write(" ".join(fields) + "\n")


def write_rows_binary(f, snapshots):
    """Binary snapshots of parsed rows (the inverse of read_result_binary)."""
    out = []
    for t, rows in snapshots:
        out.append(struct.pack("<d", t))
        for row in rows:
            out += [struct.pack("<i", row.id), row.name.encode() + b"\0", struct.pack("<i", row.type),
                    struct.pack("<4d", row.mass, row.radius, row.density, row.cd),
                    struct.pack("<i", row.mig_type), struct.pack("<7d", row.mig_stop_at, *row.r, *row.v)]
    f.write(b"".join(out))


# ------------------------------------------------------------------------------ events

def event_fields(e):
    """The 50 fields of one rg_event_t record (internal units) as the reference prints them."""
    g = T.GAUSS
    vals = [e["t"] / g, e["d"]]
    head = [EVENT_NAMES[int(e["event_name"])].rjust(16), _real(vals[0]), _real(vals[1]),
            str(int(e["id1"])).rjust(_W_INT), str(int(e["id2"])).rjust(_W_INT)]
    reals = []
    for p, r, v, oe in (("p1", "r1", "v1", "oe1"), ("p2", "r2", "v2", "oe2"), ("ps", "rs", "vs", "oes")):
        reals += [e[p]["mass"], e[p]["density"], e[p]["radius"], e[r]["x"], e[r]["y"], e[r]["z"],
                  e[v]["x"] * g, e[v]["y"] * g, e[v]["z"] * g] + [e[oe][k] for k in T.ORBELEM.names]
    return head + [_real(x) for x in reals]


def write_events(f, events):
    """rg_event_t records as the reference's event lines."""
    for e in events:
        f.write(" ".join(event_fields(e)) + " \n")


def read_event_lines(f):
    """Event lines as (name, [49 numbers as text])."""
    out = []
    for line in f:
        x = line.split()
        if x:
            out.append((x[0], x[1:]))
    return out


def write_event_lines(f, lines):
    """Lines of read_event_lines back in the reference's layout (numbers re-printed)."""
    for name, x in lines:
        head = [name.rjust(16), _real(float(x[0])), _real(float(x[1])), x[2].rjust(_W_INT), x[3].rjust(_W_INT)]
        f.write(" ".join(head + [_real(float(y)) for y in x[4:]]) + " \n")
