"""GPU SIRA with locking against the oracle's restatement of the reference's
JD-SIRA (light_locked_Huang/GEP_AB_Herm_JDSIRA_Driver4.m:12-80,
GEP_AB_Herm_JDSIRA_Locking4.m:91-505, Choose_Ritz_Pair_Unsymm4.m 'CL',
SIRA_solve_residual_LS_GEP.m:54 with SciPy MINRES for the missing minres1)
on the light-localisation inclusions at n = 8: a sphere (r = 0.25a,
gamma = 3.46427) and a regular tetrahedron (edge 0.5a, gamma = 0.5), both
called as main_EIG_np_*.m call Driver4 (target 0, 'CL', tol 1e-8, inner
MINRES tolerance 1e-2, no_restart 50).  Same eigenvalue set (1e-7
relative) and every residual within the locking rule (<= 10 tol)."""
import numpy as np
import pytest

import fame
import oracle as O
from problems import oracle_ops

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,gamma", [("sphere", 3.46427), ("tetra", 0.5)])
def test_jdsira_matches_oracle_sira(cuda, fame_lib, shape, gamma):
    n, nev, tol = 8, 6, 1e-8
    plan = fame.interior.inclusion_plan(n, [fame.fcc_point("X")], shape, gamma)
    svd, fnc, mat = oracle_ops(n, plan.thetas[0], plan.phase, plan.tensors[0])
    L = 4 * n ** 3
    fB = lambda x: O.fncB(x, fnc, mat)  # noqa: E731
    fA = lambda x: O.fncA(x, svd.Sigma_r)  # noqa: E731
    rng = np.random.default_rng(3)
    v0 = rng.random(L) + 1j * rng.random(L)
    v0 /= np.linalg.norm(v0)
    ew_o, ev_o, st = O.jdsira_driver4(fB, fA, L, 50, nev, tol, v0[:, None], 0.0, ls_tol=1e-2)
    for i in range(nev):
        assert np.linalg.norm(fB(ev_o[:, i]) - ew_o[i] * fA(ev_o[:, i])) <= 10 * tol
    r = plan.jdsira(nev, target=0.0, tol=tol, no_restart=50, restart_dim=4, inner_tol=1e-2, inner_prec="c128",
                    shift=0.0)
    assert r["status"] == 0, r
    assert np.allclose(np.sort(r["ew"]), np.sort(ew_o.real), rtol=1e-7), (np.sort(r["ew"]), np.sort(ew_o.real))
    assert np.all(r["res"] <= 10 * tol)
    plan.close()
