"""The FP64 square root and division the bit-exact gravity kernels compute on the integer
pipes (csrc/exact_fp64.h) against IEEE 754: correctly rounded, the same bits as the host's
sqrt and '/' (CPU, with the FP32 seeds perturbed) and as the GPU's sqrt.rn / div.rn on
random, near-midpoint and pair-term-like operands.  And the warp-parallel form of the serial
FP64 sum (warp_serial_sum: terms rounded to quanta of the accumulator's binade and added as
integers) against the plain serial loop, on gravity-like, wide, tie-rich, cancelling and
special-value rows."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
NATIVE = os.path.join(HERE, "native")


def _build(tmp_path, compiler, src, extra):
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    subprocess.run([compiler, *extra, "-o", exe, os.path.join(NATIVE, src)], check=True, capture_output=True,
                   text=True)
    return exe


def test_exact_sqrt_and_division_on_the_cpu(tmp_path):
    exe = _build(tmp_path, "g++", "exact_fp64_check.cpp", ["-O2", "-std=c++17", "-ffp-contract=off"])
    r = subprocess.run([exe, "200000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    bad, fb_div, fb_sqrt = map(int, re.search(r"bad (\d+) fallback_div (\d+) fallback_sqrt (\d+)", r.stdout).groups())
    assert bad == 0
    assert fb_sqrt == 0            # every positive normal operand takes the integer path
    assert fb_div < 0.1 * 7 * 5 * 200000  # only quotients outside the normal range fall back


@pytest.mark.gpu
def test_exact_sqrt_and_division_on_the_gpu(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = _build(tmp_path, nvcc, "exact_fp64_gpu.cu",
                 ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false"])
    r = subprocess.run([exe, "25"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = re.findall(r"family (\d) cases (\d+) bad (\d+) fast_div (\d+) fast_sqrt (\d+)", r.stdout)
    assert len(rows) == 5
    for fam, cases, bad, fast_div, fast_sqrt in rows:
        assert int(bad) == 0, r.stdout
        assert int(fast_sqrt) == int(cases)
        if fam != "0":  # family 0 draws exponents over the whole range, some quotients leave it
            assert int(fast_div) == int(cases)


def test_exact_serial_sum_on_the_cpu(tmp_path):
    exe = _build(tmp_path, "g++", "serial_sum_check.cpp", ["-O2", "-std=c++17", "-ffp-contract=off"])
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows, terms, bad, fast, slow, qbad = map(int, re.search(
        r"rows (\d+) terms (\d+) bad (\d+) fast (\d+) fallback (\d+) qbad (\d+)", r.stdout).groups())
    assert bad == 0 and qbad == 0
    assert terms > 7e7
    f0 = re.search(r"family 0 fast (\d+) fallback (\d+)", r.stdout)
    assert int(f0.group(1)) > 20 * int(f0.group(2))  # gravity-like rows take the integer path


@pytest.mark.gpu
def test_exact_serial_sum_on_the_gpu(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = _build(tmp_path, nvcc, "serial_sum_gpu.cu",
                 ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false"])
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = re.findall(r"family (\d) rows (\d+) bad (\d+)", r.stdout)
    assert len(rows) == 5
    assert all(int(bad) == 0 for _, _, bad in rows), r.stdout


@pytest.mark.gpu
def test_serial_sum_latency_on_the_gpu(tmp_path):
    """The warp form of the serial sum is faster than the serial FP64 loop on gravity-like
    rows (one large term, then many small ones), and no slower than twice it on rows that
    cancel, where it falls back to the serial loop; both give the same bits."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = _build(tmp_path, nvcc, "serial_sum_latency_gpu.cu",
                 ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false"])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = {int(f): (float(a), float(b), int(same)) for f, a, b, same in re.findall(
        r"family (\d) cycles per term: lane0 serial DADD ([\d.]+) \| warp_serial_sum ([\d.]+) .*same (\d)", r.stdout)}
    assert set(rows) == {0, 2, 3}, r.stdout
    assert all(v[2] == 1 for v in rows.values())
    serial, warp, _ = rows[0]
    assert warp < 0.6 * serial, r.stdout
    assert all(w < 2.0 * s_ for s_, w, _ in rows.values()), r.stdout
