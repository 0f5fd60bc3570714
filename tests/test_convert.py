"""The integer float <-> double conversions of the MIXED FP64 residual
replacement (fast_gb300/csrc/fp_convert.h): compiled as host C++
(tests/cpp/convert_check.cpp) and compared with the native conversions on
2 x 10^7 random bit patterns each way plus edge cases (zeros, the float
range's ends, rounding ties, subnormals, infinities, NaN).  Every normal
float must convert to the same bits; the documented differences (float
subnormals to a signed zero, a NaN narrowed to an infinity) are checked as
such."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_conversions_match_native(tmp_path):
    exe = str(tmp_path / "convert_check")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "fast_gb300", "csrc"),
           os.path.join(HERE, "cpp", "convert_check.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "20000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines() if line.startswith(("widen", "narrow")))
    assert lines["widen"].split() == ["20000000", "0"]
    assert lines["narrow"].split() == ["20000000", "0"]
