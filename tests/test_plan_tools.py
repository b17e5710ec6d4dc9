"""Host-side launch-plan helpers (csrc/plan_tools.h), compiled alone on the CPU."""
import os
import re
import subprocess

NATIVE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "native")


def test_symmetric_segments_cover_every_light_body_once(tmp_path):
    """build_sym_segments: the heavy-light kernel's CTAs take contiguous ranges of equal cost
    (passes of 256 light bodies + a segment cost per system start) over the light bodies of
    all systems end to end, split at system boundaries into segments of whole passes; each
    system's segments cover its light bodies once, in order, numbered as parts 1, 2, ... of
    its heavy rows (2400 cases: 1 to 300 systems of 1 to 9000 light bodies, 1 CTA to more
    CTAs than passes)."""
    exe = str(tmp_path / "sym_segments_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, os.path.join(NATIVE, "sym_segments_check.cpp")],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    cases, bad = map(int, re.search(r"cases (\d+) bad (\d+)", r.stdout).groups())
    assert cases == 2400 and bad == 0
