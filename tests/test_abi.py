"""The C-ABI library: builds, loads and exports every entry point include/*.h declares.
No computation (no GPU needed)."""
import ctypes
import os
import re

import helpers as H

HEADERS = [os.path.join(H.ROOT, "include", f) for f in os.listdir(os.path.join(H.ROOT, "include"))
           if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names.update(re.findall(r"RG_API\s+[\w\s\*]+?\b(rg_\w+)\s*\(", txt))
    return names


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "rg_create" in names and "rg_step" in names and "rg_advance" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from redgb import build, lib
    build.build()
    L = ctypes.CDLL(build.LIB)
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert missing == []
    lib.load()  # argument types bind


def test_record_sizes_match_reference_layout():
    from redgb import types as T
    assert (T.VEC.itemsize, T.PARAM.itemsize, T.BODY_MD.itemsize, T.EVENT.itemsize) == (32, 32, 24, 472)
