"""The double-single (float-float) type of csrc/fame_types.cuh on the host
(nvcc host compilation, no GPU): its additions and products within a few
units of 2^-47 of long double, near-cancelling sums included, and the
register FFT instantiated with it within 1e-13 of a direct DFT in long double
(the radix kernels and splits the double-single fncB uses)."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "3d-bi-anisotropic-phc_gb300", "csrc")


def test_double_single_arithmetic_and_fft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "ds_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", "-I", CSRC, os.path.join(HERE, "ds_host_check.cu"),
                    "-o", exe], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    lines = out.splitlines()
    m = re.match(r"arith add (\S+) mul (\S+)", lines[0])
    assert m, lines[0]
    assert float(m.group(1)) < 8 and float(m.group(2)) < 8, lines[0]
    seen = set()
    for line in lines[1:]:
        m = re.match(r"N=(\d+) fwd (\S+) inv (\S+)", line)
        assert m, line
        assert float(m.group(2)) < 1e-13 and float(m.group(3)) < 1e-13, line
        seen.add(int(m.group(1)))
    assert seen == {3, 4, 5, 12, 15, 20, 24, 40, 48, 60}
