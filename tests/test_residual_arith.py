"""The residual's rows in float-float arithmetic are as accurate as FP64 (no
GPU): a host restatement of the device arithmetic (tests/cpp/
residual_float_float.cpp) against plain double, over 60 000 random rows
covering every branch of the normal and friction projections."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "residual_float_float.cpp")


def test_float_float_residual_matches_double(tmp_path):
    exe = str(tmp_path / "residual_float_float")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", SRC, "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    m = re.search(r"scale ([0-9.e+-]+), worst sum rel err ([0-9.e+-]+); branches keep/zero/-mx/\+mx/inside "
                  r"(\d+) (\d+) (\d+) (\d+) (\d+)", out)
    assert m, out
    row_err, sum_err = float(m.group(1)), float(m.group(2))
    branches = [int(m.group(i)) for i in range(3, 8)]
    assert row_err < 1e-13 and sum_err < 1e-12, out
    assert all(b > 1000 for b in branches), out
