"""fame_restore on the GPU against the oracle's restatement of
Eigen_Restoration_Chiral_no_inv.m (fields E, H) and EvaluteError_Chiral_no_inv.m
(ORGSEP residual with the explicit sparse curl), on the same eigenvectors."""
import numpy as np
import pytest

import fame
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,label", [(6, "X"), (8, "W")])
def test_restore_matches_oracle(cuda, fame_lib, n, label):
    kvec = fame.fcc_point(label)
    plan = fame.woodpile_plan(n, [kvec])
    r = plan.lanczos(4, tol=1e-10, prec="c128")
    ev, om = r["ev"], r["omega"]
    out = plan.restore(ev, om, outside_only=False)
    out_o = plan.restore(ev, om, want_fields=False, outside_only=True)
    P = O.build_problem(n, wave_vec=kvec)
    X = ev.cpu().numpy().T
    E, H = O.eigen_restoration(X, P.fnc, P.mat)
    _, res_o = O.evaluate_error(X, om, E, H, P.dims, P.thetas, P.A, P.B, P.mat)
    Eg, Hg = out["E"].cpu().numpy().T, out["H"].cpu().numpy().T
    for j in range(4):
        scale = np.linalg.norm(np.concatenate([E[:, j], H[:, j]]))
        assert np.linalg.norm(Eg[:, j] - E[:, j]) <= 1e-12 * scale
        assert np.linalg.norm(Hg[:, j] - H[:, j]) <= 1e-12 * scale
        # the residual is a difference of O(scale * omega) terms
        assert abs(out["res_orgsep"][j] - res_o[j]) <= 1e-11 * scale * max(1.0, om[j] * n)
        Nq = n ** 3
        me = max(np.abs(E[c * Nq:(c + 1) * Nq, j]).max() for c in range(3))
        mh = max(np.abs(H[c * Nq:(c + 1) * Nq, j]).max() for c in range(3))
        assert abs(out["max_e"][j] - me) <= 1e-13 * me and abs(out["max_h"][j] - mh) <= 1e-13 * mh
        outside = ~P.inside
        me_o = max(np.abs(E[c * Nq:(c + 1) * Nq, j])[outside].max() for c in range(3))
        assert abs(out_o["max_e"][j] - me_o) <= 1e-13 * me_o
