"""The compile-time register FFT (csrc/fft_reg.cuh: Cooley-Tukey on prime
powers, prime-factor split on coprime factors) against a direct DFT for every
compiled size, evaluated on the host (nvcc host compilation, no GPU)."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "3d-bi-anisotropic-phc_gb300", "csrc")
SIZES = [4, 6, 8, 10, 12, 16, 18, 20, 24, 30, 32, 36, 40, 48, 50, 60, 64]


def test_register_fft_matches_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "fft_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", "-I", CSRC, os.path.join(HERE, "fft_host_check.cu"),
                    "-o", exe], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    seen = set()
    for line in out.splitlines():
        m = re.match(r"N=(\d+) fwd (\S+) inv (\S+)", line)
        assert m, line
        n, ef, ei = int(m.group(1)), float(m.group(2)), float(m.group(3))
        assert ef < 1e-14 and ei < 1e-14, line
        seen.add(n)
    assert seen == set(SIZES)
