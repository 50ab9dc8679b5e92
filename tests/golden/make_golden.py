"""Golden fixtures of the woodpile benchmark problem, computed by the CPU
oracle (oracle/fame_oracle.py) at sizes it finishes in seconds.

The reference is MATLAB and ships no golden vectors, so these record the
oracle's own outputs; `tests/test_golden.py` checks that the oracle still
reproduces them and `tests/test_gpu_golden.py` checks the CUDA library
against them.  Inputs are deterministic closed-form vectors (no random
generator whose stream could change between NumPy versions).

    python tests/golden/make_golden.py          # rewrites woodpile_golden.npz
    python tests/golden/make_golden.py --n24    # rewrites woodpile_n24_X.npz (~3 min)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

FILE = os.path.join(HERE, "woodpile_golden.npz")
N24_FILE = os.path.join(HERE, "woodpile_n24_X.npz")  # the first workload: n = 24, X point, 10 bands
CASES = [(4, "X"), (6, "X"), (6, "L")]   # operator fixtures
EIG_CASES = [(6, "X"), (6, "L")]          # Lanczos fixtures: k = 4, p = 8, tol 1e-10
BANDS = 4
RASTER_N = 12


def det_vec(length: int, s: int) -> np.ndarray:
    """A deterministic complex test vector."""
    j = np.arange(length, dtype=np.float64)
    return np.cos(0.731 * j + 0.37 * s) + 1j * np.sin(1.217 * j + 0.11 * s)


def images(A):
    return [A @ np.array([i, j, k], dtype=np.float64) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)]


def raster_ids(n):
    """Oracle isofunctions at the vertices of the n^3 grid (FCC, a = 1):
    woodpile width 0.25, sphere r = 0.25 and regular tetrahedron edge 0.5 at
    the origin with their periodic images."""
    A = O.fcc_lattice()
    P = O.grid_vertices(O.Dims(n, n, n)) @ A.T
    wood = O.woodpile_isofun(P, 0.25, 1.0)
    sph = O.sphere_isofun(P, np.array(images(A)), 0.25)
    s = 0.5 / (2.0 * np.sqrt(2.0))
    base = s * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64)
    tet = np.zeros(P.shape[0], dtype=bool)
    for off in images(A):
        tet |= O.tetra_isofun(P, base + off)
    return wood, sph, tet


def compute():
    out = {}
    for n, lab in CASES:
        key = f"n{n}_{lab}"
        P = O.build_problem(n, wave_vec=O.fcc_vertex(lab))
        Nq = n ** 3
        x = det_vec(4 * Nq, n)
        y3 = det_vec(3 * Nq, n + 1)
        out[key + "_theta"] = np.asarray(P.thetas, dtype=np.float64)
        out[key + "_inside"] = P.inside.astype(np.uint8)
        out[key + "_Bx"] = O.fncB(x, P.fnc, P.mat)
        out[key + "_Ax"] = P.A(x)
        out[key + "_Tn"] = O.mtxvecmul_fft(y3, P.dims, "notranspose", P.svd.S, P.svd.D)
        out[key + "_Tt"] = O.mtxvecmul_fft(y3, P.dims, "transpose", P.svd.S, P.svd.D)
    for n, lab in EIG_CASES:
        P = O.build_problem(n, wave_vec=O.fcc_vertex(lab))
        L = 4 * n ** 3
        _, ew, _ = O.lanczos(P.A, P.B, lambda r: O.fncinvB(r, P.B, 1e-12, 10000), L, BANDS, 1e-10, 10000,
                             2 * BANDS, np.ones(L, complex))
        out[f"n{n}_{lab}_ew"] = np.asarray(ew, dtype=np.float64)
    wood, sph, tet = raster_ids(RASTER_N)
    out["raster_woodpile"] = np.packbits(wood)
    out["raster_sphere"] = np.packbits(sph)
    out["raster_tetra"] = np.packbits(tet)
    return out


def compute_n24(k=10):
    """The woodpile at n = 24 and the X point, the 10 largest eigenvalues of
    B^-1 A by the oracle's Lanczos.m (p = 2k, tol 1e-10, inner pcg 1e-12)."""
    P = O.build_problem(24, wave_vec=O.fcc_vertex("X"))
    L = 4 * 24 ** 3
    _, ew, it = O.lanczos(P.A, P.B, lambda r: O.fncinvB(r, P.B, 1e-12, 10000), L, k, 1e-10, 10000, 2 * k,
                          np.ones(L, complex))
    return {"ew": np.asarray(ew, dtype=np.float64), "theta": np.asarray(P.thetas, dtype=np.float64)}


if __name__ == "__main__":
    if "--n24" in sys.argv:
        np.savez_compressed(N24_FILE, **compute_n24())
        print("wrote", N24_FILE, os.path.getsize(N24_FILE), "bytes")
    else:
        np.savez_compressed(FILE, **compute())
        print("wrote", FILE, os.path.getsize(FILE), "bytes")
