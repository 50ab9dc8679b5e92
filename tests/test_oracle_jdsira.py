"""The oracle's restatement of JD-SIRA with locking
(light_locked_Huang/GEP_AB_Herm_JDSIRA_Driver4.m, _Locking4.m,
Choose_Ritz_Pair_Unsymm4.m 'CL', SIRA_solve_residual_LS_GEP.m with SciPy
MINRES for the missing minres1) against the dense spectrum of the oracle's
operators at n = 4: the eigenvalues above the target, closest first, with
the locking rule's residuals (rsdl <= tol, or <= 10 tol after five steps)."""
import numpy as np
import pytest
import scipy.linalg as sla

import oracle as O


def dense_thetas(P, n):
    L = 4 * n ** 3
    I = np.eye(L, dtype=complex)
    B = np.stack([P.B(I[:, j]) for j in range(L)], axis=1)
    A = np.stack([P.A(I[:, j]) for j in range(L)], axis=1)
    mu = sla.eigh(0.5 * (A + A.conj().T), 0.5 * (B + B.conj().T), eigvals_only=True)
    return 1.0 / mu


@pytest.mark.parametrize("target,gamma,shift", [(0.0, 0.2, 0.0), (6.0, 0.5, 6.0)])
def test_oracle_jdsira_matches_dense(target, gamma, shift):
    n, nev, tol = 4, 5, 1e-8
    P = O.build_problem(n, wave_vec=O.fcc_vertex("X"), gamma=gamma)
    L = 4 * n ** 3
    th = dense_thetas(P, n)
    rng = np.random.default_rng(0)
    v0 = rng.random(L) + 1j * rng.random(L)
    v0 /= np.linalg.norm(v0)
    # Driver4(fncB, fncA, ...): A := fncB, B := fncA
    ew, ev, st = O.jdsira_driver4(P.B, P.A, L, 30, nev, tol, v0[:, None], target, shift=shift)
    assert np.allclose(np.sort(ew.real), np.sort(th[th > target])[:nev], rtol=1e-9)
    for i in range(nev):
        assert np.linalg.norm(P.B(ev[:, i]) - ew[i] * P.A(ev[:, i])) <= 10 * tol
    assert st["outer"] > 0 and st["minres"] > 0


def test_gram_schmidt_drops_dependent_columns():
    rng = np.random.default_rng(1)
    Y = rng.standard_normal((20, 3)) + 1j * rng.standard_normal((20, 3))
    Y = np.concatenate([Y, Y[:, :1] * 2.0], axis=1)
    Q = O.gram_schmidt_ref(Y)
    assert Q.shape[1] == 3
    assert np.allclose(Q.conj().T @ Q, np.eye(3), atol=1e-12)
