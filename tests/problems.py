"""Paired test problems: the same inputs built for the CUDA library (product)
and for the CPU oracle (checker)."""
from __future__ import annotations

import numpy as np

import fame
import oracle as O


def random_tensors(rng, nphase, hermitian=True):
    """Per-phase covariant N, M, J blocks (27 complex).  Hermitian N, M
    diagonal-dominant blocks with a weak J mimic physical materials (B is then
    positive definite, as CG needs); hermitian=False gives general complex
    blocks (exercises the (X+X')/2 symmetrisation)."""
    out = np.zeros((nphase, 27), dtype=np.complex128)
    for p in range(nphase):
        for b in range(3):
            m = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3))
            if hermitian and b < 2:
                m = 0.5 * (m + m.conj().T) * 0.2 + np.eye(3) * (1.0 + p)
            elif hermitian:
                m = 0.1 * m  # weak coupling keeps [M J'; J N] positive definite
            out[p, b * 9:(b + 1) * 9] = m.ravel()
    return out


def oracle_ops(n, thetas, phase, tens):
    """Oracle BandProblem pieces for one instance with per-phase tensors
    `tens` (nphase x 27)."""
    dims = O.Dims(n, n, n)
    svd = O.svd_matrix_generate(dims, thetas)
    fnc = O.make_handles(svd)

    def vert(blk):
        t = tens[:, blk * 9:(blk + 1) * 9].reshape(-1, 3, 3)
        return [[t[phase, i, j] for j in range(3)] for i in range(3)]

    Nint, Mint, Jint = O.interp_material_vertex(dims, thetas, vert(0), vert(1), vert(2))
    mat = O.MaterialOps(Nint, Mint, Jint)
    return svd, fnc, mat


class Pair:
    def __init__(self, n, nk=2, seed=0, hermitian=True, nphase=2, thetas=None):
        rng = np.random.default_rng(seed)
        self.n = n
        self.Nq = n ** 3
        if thetas is None:
            thetas = rng.uniform(-np.pi, np.pi, size=(nk, 3))
        self.thetas = np.asarray(thetas, dtype=np.float64).reshape(-1, 3)
        self.nk = self.thetas.shape[0]
        self.phase = rng.integers(0, nphase, size=self.Nq).astype(np.uint8)
        self.tens = np.stack([random_tensors(rng, nphase, hermitian) for _ in range(self.nk)])
        self.plan = fame.Plan(n, self.thetas, self.phase, self.tens)
        self._ref = {}
        self.rng = rng

    def ref(self, k):
        if k not in self._ref:
            self._ref[k] = oracle_ops(self.n, tuple(self.thetas[k]), self.phase, self.tens[k])
        return self._ref[k]

    def vec(self, L, nvec=None):
        shape = (L,) if nvec is None else (nvec, L)
        return self.rng.standard_normal(shape) + 1j * self.rng.standard_normal(shape)


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))
