"""The oracle's restatement of subroutines/Lanczos_gep.m at n = 4 against the
dense spectrum: with the B-norm restart scaling it converges to the k largest
|lambda| of B^{-1}A; the literal Euclidean scaling of Lanczos_gep.m:77 leaves
the basis non-B-orthonormal after the first restart."""
import numpy as np
import scipy.linalg as sla

import oracle as O


def dense(n=4):
    P = O.build_problem(n, wave_vec=O.fcc_vertex("X"))
    L = 4 * n ** 3
    I = np.eye(L, dtype=complex)
    B = np.stack([P.B(I[:, j]) for j in range(L)], axis=1)
    A = np.stack([P.A(I[:, j]) for j in range(L)], axis=1)
    B = 0.5 * (B + B.conj().T)
    A = 0.5 * (A + A.conj().T)
    return P, A, B, L


def test_lanczos_gep_bnorm_matches_dense():
    P, A, B, L = dense()
    mu = sla.eigh(A, B, eigvals_only=True)
    Binv = np.linalg.inv(B)
    w = np.ones(L, complex)
    v0 = w / np.sqrt(np.vdot(w, P.B(w)).real)
    k = 6
    EV, EW, nit = O.lanczos_gep(P.A, P.B, lambda r: Binv @ r, L, k, 14, 500, 1e-10, v0, bnorm_restart=True)
    assert EV is not None
    ref = np.sort(mu[np.argsort(-np.abs(mu))][:k])
    assert np.allclose(np.sort(EW), ref, rtol=1e-10)
    for j in range(k):
        x = EV[:, j]
        assert np.linalg.norm(P.A(x) - EW[j] * P.B(x)) <= 1e-9 * np.linalg.norm(x)


def test_lanczos_gep_literal_restart_loses_b_orthonormality():
    P, A, B, L = dense()
    Binv = np.linalg.inv(B)
    w = np.ones(L, complex)
    v0 = w / np.sqrt(np.vdot(w, P.B(w)).real)
    EV, EW, nit = O.lanczos_gep(P.A, P.B, lambda r: Binv @ r, L, 6, 14, 500, 1e-10, v0)
    assert EV is not None  # the stopping test is met ...
    res = [np.linalg.norm(P.A(EV[:, j]) - EW[j] * P.B(EV[:, j])) / np.linalg.norm(EV[:, j]) for j in range(6)]
    assert max(res) > 1e-6  # ... with pairs that are not eigenpairs
