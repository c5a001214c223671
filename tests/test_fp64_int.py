"""The integer-pipe FP64 helpers (gpuvoxels_gb300/csrc/fp64_int.cuh) return bit-for-bit
what the FP64 instructions they replace return: checked on the host against IEEE-754
arithmetic over random bit patterns, rounding ties, exponent boundaries and the special
values (tests/fp64_int_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fp64_integer_helpers_match_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "fp64_int_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "fp64_int_check.cpp")],
                   check=True)
    r = subprocess.run([exe, "6000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
