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


def test_generator_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the initial-condition structs have the header's sizes and field
    offsets (a small C++ program compiled against include/redgb_types.h prints them)."""
    import shutil
    import subprocess
    import pytest
    from redgb import icgen
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    src = tmp_path / "layout.cpp"
    src.write_text("""
#include <cstddef>
#include <cstdio>
#include "redgb_types.h"
#define P(T, f) std::printf("%s.%s %zu\\\\n", #T, #f, offsetof(T, f));
int main() {
    std::printf("rg_dist_t %zu\\\\nrg_body_disk_t %zu\\\\nrg_mmsn_component_t %zu\\\\nrg_disk_spec_t %zu\\\\n",
                sizeof(rg_dist_t), sizeof(rg_body_disk_t), sizeof(rg_mmsn_component_t), sizeof(rg_disk_spec_t));
    P(rg_dist_t, p) P(rg_body_disk_t, n_body) P(rg_body_disk_t, to_bc) P(rg_body_disk_t, pp_total_mass)
    P(rg_body_disk_t, oe) P(rg_body_disk_t, pp) P(rg_mmsn_component_t, p)
    P(rg_disk_spec_t, giant_m) P(rg_disk_spec_t, m_lo) P(rg_disk_spec_t, a_mode) P(rg_disk_spec_t, sigma_e)
    P(rg_disk_spec_t, rho_pl)
    return 0;
}
""".replace("\\\\n", "\\n"))
    exe = tmp_path / "layout"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(H.ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.split("\n") if line)
    got = {k: int(v) for k, v in got.items()}
    assert got["rg_dist_t"] == ctypes.sizeof(icgen.DistC)
    assert got["rg_body_disk_t"] == ctypes.sizeof(icgen.BodyDiskC)
    assert got["rg_mmsn_component_t"] == ctypes.sizeof(icgen.MmsnC)
    assert got["rg_disk_spec_t"] == ctypes.sizeof(icgen.DiskSpecC)
    for cname, cls in (("rg_dist_t", icgen.DistC), ("rg_body_disk_t", icgen.BodyDiskC),
                       ("rg_mmsn_component_t", icgen.MmsnC), ("rg_disk_spec_t", icgen.DiskSpecC)):
        for key, off in got.items():
            if key.startswith(cname + "."):
                assert getattr(cls, key.split(".", 1)[1]).offset == off, key


def test_every_mirrored_struct_matches_the_header(tmp_path):
    """Sizes of all C structs the Python view mirrors (ctypes classes and numpy records)."""
    import shutil
    import subprocess
    import pytest
    from redgb import types as T
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    names = ["rg_vec_t", "rg_param_t", "rg_body_metadata_t", "rg_orbelem_t", "rg_event_t", "rg_counts_t",
             "rg_counters_t", "rg_profile_t", "rg_tune_t", "rg_ens_stats_t", "rg_step_rec_t"]
    src = tmp_path / "sizes.cpp"
    body = "".join(f'    std::printf("{n} %zu\\n", sizeof({n}));\n' for n in names)
    src.write_text('#include <cstdio>\n#include "redgb_types.h"\nint main() {\n' + body + "    return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(H.ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {k: int(v) for k, v in (line.split() for line in
                                  subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())}
    mirrors = {"rg_vec_t": T.VEC.itemsize, "rg_param_t": T.PARAM.itemsize, "rg_body_metadata_t": T.BODY_MD.itemsize,
               "rg_orbelem_t": T.ORBELEM.itemsize, "rg_event_t": T.EVENT.itemsize,
               "rg_counts_t": ctypes.sizeof(T.Counts), "rg_counters_t": ctypes.sizeof(T.Counters),
               "rg_profile_t": ctypes.sizeof(T.Profile), "rg_tune_t": ctypes.sizeof(T.Tune),
               "rg_ens_stats_t": ctypes.sizeof(T.EnsStats), "rg_step_rec_t": T.STEP_REC.itemsize}
    assert got == mirrors


def test_energy_noalloc_host_checks_without_a_device():
    """rg_energy_noalloc's argument checks run on the host before any device work, so they
    are exercised here without a GPU: no bodies gives zeros; a negative count, a missing
    body array with bodies to read, or more bodies than its fixed scratch holds give
    RG_ERR_ARG."""
    from redgb import lib, types as T
    L = lib.load()
    f = L.rg_energy_noalloc
    vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
    f.argtypes = [ctypes.POINTER(T.Counts), vp, vp, vp, vp, vp, dp, dp]
    f.restype = ctypes.c_int
    RG_ERR_ARG = -1

    def call(counts, arrays=(None, None, None, None)):
        e = ctypes.c_double(123.0)
        Lm = (ctypes.c_double * 3)(1.0, 2.0, 3.0)
        rc = f(ctypes.byref(counts) if counts is not None else None, *arrays, None, ctypes.byref(e), Lm)
        return rc, e.value, list(Lm)

    assert call(T.Counts()) == (0, 0.0, [0.0, 0.0, 0.0])
    assert call(None)[0] == RG_ERR_ARG
    neg = T.Counts()
    neg.n_s, neg.n_pl = 1, -2
    assert call(neg)[0] == RG_ERR_ARG and "negative" in L.rg_last_error().decode()
    some = T.Counts()
    some.n_s, some.n_pl = 1, 10
    fake = ctypes.c_void_p(16)  # never dereferenced: a missing array is refused first
    for k in range(4):
        arrays = [fake] * 4
        arrays[k] = None
        assert call(some, arrays)[0] == RG_ERR_ARG and "null body array" in L.rg_last_error().decode()
    big = T.Counts()
    big.n_s, big.n_pl = 1, 65536
    assert call(big)[0] == RG_ERR_ARG and "65536" in L.rg_last_error().decode()
