"""The mixed engine's integer-pipe FP32 <-> FP64 conversions (csrc/swc_fpconv.h) give the
same bits as the C casts (CPU build of the same header)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(__file__)
CSRC = os.path.join(HERE, "..", "smaiso_wcomp_gb300", "csrc")


def test_conversions_match_casts(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = os.path.join(tmp_path, "fpconv_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "fpconv_check.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout


def test_fp64_reciprocal_within_an_ulp(tmp_path):
    """rcp_f64, the FP64 engine's Newton-Raphson reciprocal: within one ulp of the IEEE
    division from seeds 2^-20 off, and the division itself outside its range."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = os.path.join(tmp_path, "rcp_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, os.path.join(HERE, "rcp_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "rcp mismatches 0" in r.stdout
