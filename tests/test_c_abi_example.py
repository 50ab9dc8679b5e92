"""include/fame.h is a plain C interface: tests/c_abi_example.c (a C99 caller
doing what a MEX gateway does for the woodpile problem) compiles with
-Wall -Wextra -Werror and links against the library; without a GPU it fails
loudly (no CPU fallback); on the GPU its FP64 eigenvalues equal the golden
fixture's (the oracle's Lanczos.m)."""
import os
import subprocess

import numpy as np
import pytest

import fame
from golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_example(tmp_path):
    libdir = os.path.dirname(fame.lib_path())
    exe = str(tmp_path / "c_abi_example")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "c_abi_example.c"), "-L", libdir, "-lfame_gb300", f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_caller_compiles_and_links(fame_lib, tmp_path):
    assert os.path.exists(build_example(tmp_path))


def test_c_caller_fails_loudly_without_gpu(fame_lib, tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([build_example(tmp_path), "6", "4"], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "failed" in r.stderr


@pytest.mark.gpu
def test_c_caller_matches_golden_eigenvalues(cuda, fame_lib, tmp_path):
    r = subprocess.run([build_example(tmp_path), "6", str(G.BANDS)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    ew = np.array([float(v) for v in lines[:G.BANDS]])
    ref = np.load(G.FILE)["n6_X_ew"]
    assert np.allclose(ew, ref, rtol=1e-10, atol=0), (ew, ref)
    assert float(lines[G.BANDS].split()[1]) < 1e-8
