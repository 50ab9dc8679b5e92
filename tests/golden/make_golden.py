"""Golden fixtures of the woodpile benchmark problem, computed by the CPU
oracle (oracle/fame_oracle.py) at sizes it finishes in seconds.

The reference is MATLAB and ships no golden vectors, so these record the
oracle's own outputs; `tests/test_golden.py` checks that the oracle still
reproduces them and `tests/test_gpu_golden.py` checks the CUDA library
against them.  Inputs are deterministic closed-form vectors (no random
generator whose stream could change between NumPy versions).

    python tests/golden/make_golden.py          # rewrites woodpile_golden.npz
    python tests/golden/make_golden.py --n24    # rewrites woodpile_n24_X.npz (~3 min)
    python tests/golden/make_golden.py --n60ops # operator digests at n = 60 (~1 min)
    python tests/golden/make_golden.py --n60eig # FP64 Lanczos at n = 60, X (~40 min)

At n = 60 one complex128 vector is 13.8 MB, so the n = 60 fixtures keep a
digest of each output instead of the vector: its values at 1024 fixed
indices, its inner products with four closed-form sketch vectors, and its
norm (`digest`).  A wrong entry anywhere changes the sketches; the sampled
values localise it.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

FILE = os.path.join(HERE, "woodpile_golden.npz")
N24_FILE = os.path.join(HERE, "woodpile_n24_X.npz")  # the first workload: n = 24, X point, 10 bands
N60_OPS_FILE = os.path.join(HERE, "woodpile_n60_ops.npz")  # operator digests at the benchmark size
N60_EIG_FILE = os.path.join(HERE, "woodpile_n60_X.npz")    # FP64 eigenvalues at the benchmark size
N60_LABELS = ("X", "L")
N60_SAMPLES = 1024
N60_SKETCHES = 4
CASES = [(4, "X"), (6, "X"), (6, "L")]   # operator fixtures
EIG_CASES = [(6, "X"), (6, "L")]          # Lanczos fixtures: k = 4, p = 8, tol 1e-10
BANDS = 4
RASTER_N = 12


def det_vec(length: int, s: int) -> np.ndarray:
    """A deterministic complex test vector."""
    j = np.arange(length, dtype=np.float64)
    return np.cos(0.731 * j + 0.37 * s) + 1j * np.sin(1.217 * j + 0.11 * s)


def sample_index(length: int) -> np.ndarray:
    """The fixed indices a digest samples (a stride coprime to every vector length used)."""
    return np.unique((np.arange(N60_SAMPLES, dtype=np.int64) * 104729 + 17) % length)


def digest(y: np.ndarray) -> dict:
    """Sampled values, sketch inner products <s_j, y> and the norm of y."""
    y = np.asarray(y, dtype=np.complex128).ravel()
    L = y.shape[0]
    sk = np.array([np.vdot(det_vec(L, 1000 + j), y) for j in range(N60_SKETCHES)])
    return {"samp": y[sample_index(L)], "sketch": sk, "norm": np.array([np.linalg.norm(y)])}


def digest_relerr(y: np.ndarray, ref: dict) -> float:
    """Largest relative deviation of y's digest from a stored one (each part
    relative to the reference's own scale: ||samples||, ||s_j||*||y||, ||y||)."""
    d = digest(y)
    L = np.asarray(y).size
    e1 = np.linalg.norm(d["samp"] - ref["samp"]) / np.linalg.norm(ref["samp"])
    e2 = np.max(np.abs(d["sketch"] - ref["sketch"])) / (np.sqrt(L) * ref["norm"][0])
    e3 = abs(d["norm"][0] - ref["norm"][0]) / ref["norm"][0]
    return float(max(e1, e2, e3))


def n60_ops_inputs(n: int = 60):
    Nq = n ** 3
    return det_vec(4 * Nq, n), det_vec(3 * Nq, n + 1)


N60_OPS = ("Bx", "Ax", "Tn", "Tt", "Pr", "Qr", "Prs", "Qrs")


def compute_n60_ops(n: int = 60):
    """fncB, fncA, MtxVecMul_FFT both ways and the Pr/Qr/Prs/Qrs handles of the
    woodpile at n = 60 (X and L), as digests."""
    out = {}
    x, y3 = n60_ops_inputs(n)
    Nq = n ** 3
    for lab in N60_LABELS:
        P = O.build_problem(n, wave_vec=O.fcc_vertex(lab))
        outs = {
            "Bx": P.B(x), "Ax": P.A(x),
            "Tn": O.mtxvecmul_fft(y3, P.dims, "notranspose", P.svd.S, P.svd.D),
            "Tt": O.mtxvecmul_fft(y3, P.dims, "transpose", P.svd.S, P.svd.D),
            "Pr": P.fnc.Pr(x[:2 * Nq]), "Qr": P.fnc.Qr(x[2 * Nq:]),
            "Prs": P.fnc.Prs(y3), "Qrs": P.fnc.Qrs(y3),
        }
        out[f"{lab}_theta"] = np.asarray(P.thetas, dtype=np.float64)
        for name, y in outs.items():
            for part, v in digest(y).items():
                out[f"{lab}_{name}_{part}"] = v
    return out


def n60_ref(fix, lab: str, name: str) -> dict:
    return {part: fix[f"{lab}_{name}_{part}"] for part in ("samp", "sketch", "norm")}


def compute_n60_eig(k=10):
    """The woodpile at n = 60 and the X point: the 10 largest eigenvalues of
    B^-1 A by the oracle's Lanczos.m (p = 2k, tol 1e-10, inner pcg 1e-12),
    as band_structure_woodpile_Lanczos_n60_gamma0p2.m:74-81 runs each k-point."""
    O.fft_workers(os.cpu_count() or 1)
    P = O.build_problem(60, wave_vec=O.fcc_vertex("X"))
    L = 4 * 60 ** 3
    nits = []
    nB = [0]

    def fB(x):
        nB[0] += 1
        return P.B(x)

    t0 = time.perf_counter()
    _, ew, it = O.lanczos(P.A, fB, lambda r: O.fncinvB(r, fB, 1e-12, 10000, stats=nits), L, k, 1e-10, 10000,
                          2 * k, np.ones(L, complex))
    return {"ew": np.asarray(ew, dtype=np.float64), "theta": np.asarray(P.thetas, dtype=np.float64),
            "lanczos_steps": np.array([it]), "pcg_iters": np.array([int(np.sum(nits))]),
            "b_applies": np.array([nB[0]]), "seconds": np.array([time.perf_counter() - t0]),
            "cpu_threads": np.array([O.fft_workers()])}


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
    if "--n60ops" in sys.argv:
        np.savez_compressed(N60_OPS_FILE, **compute_n60_ops())
        print("wrote", N60_OPS_FILE, os.path.getsize(N60_OPS_FILE), "bytes")
    elif "--n60eig" in sys.argv:
        np.savez_compressed(N60_EIG_FILE, **compute_n60_eig())
        print("wrote", N60_EIG_FILE, os.path.getsize(N60_EIG_FILE), "bytes")
    elif "--n24" in sys.argv:
        np.savez_compressed(N24_FILE, **compute_n24())
        print("wrote", N24_FILE, os.path.getsize(N24_FILE), "bytes")
    else:
        np.savez_compressed(FILE, **compute())
        print("wrote", FILE, os.path.getsize(FILE), "bytes")
