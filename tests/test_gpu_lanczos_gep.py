"""fame.Lanczos_gep (subroutines/Lanczos_gep.m on the GPU handles) against
the oracle's line-by-line restatement on the same start vector: with the
B-norm restart scaling both converge to the same eigenvalues; with the
reference's literal Euclidean scaling both take the same iterations."""
import numpy as np
import pytest

import fame
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bnorm,rtol", [(True, 1e-10), (False, 1e-6)])
def test_lanczos_gep_matches_oracle(cuda, fame_lib, bnorm, rtol):
    n, k, m = 6, 4, 10
    kvec = fame.fcc_point("W")
    P = O.build_problem(n, wave_vec=kvec)
    L = 4 * n ** 3
    w = np.ones(L, complex)
    v0 = w / np.sqrt(np.vdot(w, P.B(w)).real)
    EVo, EWo, nito = O.lanczos_gep(P.A, P.B, lambda r: O.fncinvB(r, P.B, 1e-12, 10000), L, k, m, 300, 1e-10, v0,
                                   bnorm_restart=bnorm)
    plan = fame.woodpile_plan(n, [kvec])
    EV, EW, nit = fame.Lanczos_gep(plan, k, dict(m=m, itmax=300, tol=1e-10, v0=v0, bnorm=bnorm))
    assert EV is not None and EVo is not None
    assert nit == nito
    assert np.allclose(np.sort(EW), np.sort(EWo), rtol=rtol, atol=0)
    if bnorm:
        ax = plan.apply_A(EV).cpu().numpy()
        bx = plan.apply_B(EV).cpu().numpy()
        for j in range(k):
            assert np.linalg.norm(ax[j] - EW[j] * bx[j]) <= 1e-8 * np.linalg.norm(EV[j].cpu().numpy())
