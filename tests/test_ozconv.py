"""CPU check (no GPU): the 64-bit FP64 conversion used by the tensor-core linear
combination's drain equals the general 128-bit conversion bit for bit, over
random level vectors, rounding ties and the exponent-range fallback."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gcge-1.0_gb300", "csrc")


def test_oz_to_double40_matches_general_form(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "ozconv_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "ozconv_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
