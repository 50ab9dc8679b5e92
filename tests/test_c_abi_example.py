"""include/fame.h is a plain C interface: tests/c_abi_example.c (a C99 caller
doing what a MEX gateway does for the woodpile problem) compiles with
-Wall -Wextra -Werror and links against the library; without a GPU it fails
loudly (no CPU fallback); on the GPU its FP64 eigenvalues equal the golden
fixture's (the oracle's Lanczos.m), and its backward-entry mode
(fame_plan_create_field, fame_lanczos, fame_eig_gradient) gives the oracle's
FP64 reference gradient of the band-2/3 gap (dense solve at n = 6)."""
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
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cudalib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                                os.path.join(cuda, "targets", "x86_64-linux", "lib")) if os.path.isdir(d)),
                   os.path.join(cuda, "lib64"))
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(HERE, "c_abi_example.c"), "-L", libdir,
           "-lfame_gb300", f"-Wl,-rpath,{libdir}", "-L", cudalib, "-lcudart", f"-Wl,-rpath,{cudalib}", "-lm",
           "-o", exe]
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


@pytest.mark.gpu
def test_c_caller_gradient_matches_oracle(cuda, fame_lib, tmp_path):
    import scipy.linalg as sla

    import oracle as O

    n, k = 6, 4
    r = subprocess.run([build_example(tmp_path), "grad", str(n), str(k)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    om = np.array([float(v) for v in lines[:k]])
    g = np.array([[float(t) for t in ln.split()[1:]] for ln in lines[k:]])
    assert g.shape == (n ** 3, 2)
    # the same field and k-point through the oracle: dense FP64 eigenpairs and
    # the reference gradient of omega_3 - omega_2
    i1, i2, i3 = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    s = ((73 * i1 + 151 * i2 + 37 * i3 + 11) % 97) / 96.0
    s = s.transpose(2, 1, 0).ravel()  # x fastest
    eps, gam = 1.0 + 12.0 * s, 0.2 * s
    P = O.build_problem_field(n, eps, gam, thetas=(np.pi, 0.0, np.pi))
    L = 4 * n ** 3
    I = np.eye(L, dtype=complex)
    Bm = np.stack([P.B(I[:, j]) for j in range(L)], axis=1)
    Am = np.stack([P.A(I[:, j]) for j in range(L)], axis=1)
    lam, X = sla.eigh(0.5 * (Am + Am.conj().T), 0.5 * (Bm + Bm.conj().T))
    order = np.argsort(-lam)[:k]  # the k largest lambda = 1/omega, as Lanczos.m
    assert np.allclose(om, 1.0 / lam[order], rtol=1e-10)
    assert abs(lam[order[1]] - lam[order[2]]) > 1e-6 * abs(lam[order[1]])  # bands 2, 3 not degenerate
    ge = np.zeros(n ** 3)
    gg = np.zeros(n ** 3)
    for b, wb in ((1, -1.0), (2, 1.0)):
        e_, g_, _ = O.field_gradient(P, X[:, order[b]], 1.0 / lam[order[b]], eps, gam)
        ge += wb * e_
        gg += wb * g_
    assert np.linalg.norm(g[:, 0] - ge) <= 1e-6 * np.linalg.norm(ge)
    assert np.linalg.norm(g[:, 1] - gg) <= 1e-6 * np.linalg.norm(gg)
