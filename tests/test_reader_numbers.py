"""The VXA reader's number fields (PhaseOffset, cilia force layers) are read with
gvx::field_atof; it must give atof's double bit for bit (tests/field_atof_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "gpuvoxels_gb300", "csrc")


def test_field_atof_matches_atof(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "field_atof_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, "-I", os.path.join(HERE, "..", "include"), "-o", exe,
                    os.path.join(HERE, "field_atof_check.cpp"), os.path.join(CSRC, "world.cpp"),
                    os.path.join(CSRC, "xml_dom.cpp"), "-lpthread"], check=True)
    r = subprocess.run([exe, "300000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
