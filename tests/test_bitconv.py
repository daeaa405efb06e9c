"""The integer-pipe binary64 <-> binary32 conversions of the cell kernels
(hydro_rs_gb300/csrc/bitconv.cuh), built as host C++ and checked against the
compiler's IEEE casts: round to nearest even, subnormal results, overflow,
exact halfway cases, every binary32 subnormal.  (The device build of the same
header is checked against the GPU's own conversion instructions through the
FP32-face parity tests.)"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bitconv_matches_ieee_casts(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "bitconv_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "bitconv_check.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
