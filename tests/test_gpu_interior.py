"""Shifted SIRA on inclusion crystals (the light-localisation configuration of
main_EIG_np_sphere_n60_gamma3p46427.m / main_EIG_np_tri_n60_gamma*.m, with the
target at 1.05x the 4th band edge at Gamma): eigenvalues against the dense
spectrum of the oracle's operators at n = 6, field maxima from fame_restore."""
import numpy as np
import pytest
import scipy.linalg as sla

import fame
import oracle as O
from problems import oracle_ops

pytestmark = pytest.mark.gpu


def dense_omegas(plan, n):
    """Dense spectrum of fncB x = omega fncA x for instance 0 of `plan`
    (the oracle's literal operators with the plan's phases and tensors)."""
    svd, fnc, mat = oracle_ops(n, plan.thetas[0], plan.phase, plan.tensors[0])
    L = 4 * n ** 3
    I = np.eye(L, dtype=complex)
    B = np.stack([O.fncB(I[:, j], fnc, mat) for j in range(L)], axis=1)
    A = np.stack([O.fncA(I[:, j], svd.Sigma_r) for j in range(L)], axis=1)
    mu = sla.eigh(0.5 * (A + A.conj().T), 0.5 * (B + B.conj().T), eigvals_only=True)
    return 1.0 / mu


@pytest.mark.parametrize("shape,gamma", [("sphere", 3.46427), ("tetra", 0.5), ("tetra", 1.009)])
def test_interior_modes_match_dense(cuda, fame_lib, shape, gamma):
    n, nev = 6, 4
    plan = fame.interior.inclusion_plan(n, [np.zeros(3)], shape, gamma)
    om = dense_omegas(plan, n)
    pos = np.sort(om[om > 0])
    sigma = 1.05 * pos[3]
    assert abs(fame.interior.band_edge(plan, prec="c128") - pos[3]) <= 1e-9 * pos[3]
    ref = om[np.argsort(np.abs(om - sigma))][:nev]
    r = fame.interior.interior_modes(plan, nev, sigma, tol=1e-8, inner_tol=1e-3)
    assert r["status"] == 0, r["status"]
    assert np.allclose(np.sort(r["omega"]), np.sort(ref), rtol=1e-7), (np.sort(r["omega"]), np.sort(ref))
    assert np.all(r["res_nfsep"] <= 1e-7)
    assert np.all(np.isfinite(r["max_e"])) and np.all(r["max_e"] > 0) and np.all(r["max_h"] > 0)
