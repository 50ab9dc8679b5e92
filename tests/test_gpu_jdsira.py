"""SIRA with locking (GEP_AB_Herm_JDSIRA_Driver4.m as called in main_EIG_np_*.m:
Driver4(fncB, fncA, ...)) on the GPU: the eigenvalues of fncB x = theta fncA x
closest to a target must be the exact ones of the oracle's operators (dense
spectrum at n = 4), with the requested residual."""
import numpy as np
import pytest
import scipy.linalg as sla

import fame
import oracle as O

pytestmark = pytest.mark.gpu


def dense_thetas(n, kvec, gamma):
    P = O.build_problem(n, wave_vec=kvec, gamma=gamma)
    Lv = 4 * n ** 3
    I = np.eye(Lv, dtype=complex)
    B = np.stack([P.B(I[:, j]) for j in range(Lv)], axis=1)
    A = np.stack([P.A(I[:, j]) for j in range(Lv)], axis=1)
    B = 0.5 * (B + B.conj().T)
    A = 0.5 * (A + A.conj().T)
    mu = sla.eigh(A, B, eigvals_only=True)  # A x = mu B x, theta = 1/mu
    return 1.0 / mu


@pytest.mark.parametrize("target,gamma", [(0.0, 0.2), (6.0, 0.5)])
@pytest.mark.parametrize("inner_prec", ["c64", "c128"])
def test_jdsira_matches_dense_spectrum(cuda, fame_lib, target, gamma, inner_prec):
    n, nev = 4, 5
    kvec = fame.fcc_point("X")
    th = dense_thetas(n, kvec, gamma)
    # 'CL' (Choose_Ritz_Pair_Unsymm4.m:176-186): the eigenvalues above the target, closest first
    above = np.sort(th[th > target])
    ref = above[:nev]
    plan = fame.woodpile_plan(n, [kvec], gamma=gamma)
    # the reference's correction drops the shift (fine for target 0); an interior
    # target uses the shifted correction
    r = plan.jdsira(nev, target=target, tol=1e-8, no_restart=30, restart_dim=4, inner_tol=1e-2,
                    inner_prec=inner_prec, want_vectors=True, shift=target)
    assert r["status"] == 0, r
    got = np.sort(r["ew"])
    assert np.allclose(got, np.sort(ref), rtol=1e-7, atol=1e-9), (got, np.sort(ref))
    # Locking4.m:198-208 accepts a pair at rsdl <= tol, or after five consecutive
    # steps with tol < rsdl <= 10 tol
    assert np.all(r["res"] <= 1e-7)
    # returned vectors are unit eigenvectors: ||B u - theta A u|| small
    ev = r["ev"]
    bu = plan.apply_B(ev).cpu().numpy()
    au = plan.apply_A(ev).cpu().numpy()
    for i in range(nev):
        assert np.linalg.norm(bu[i] - r["ew"][i] * au[i]) < 1e-7


def test_jdsira_graph_modes_agree(cuda, fame_lib):
    """The shifted MINRES of the correction equation run as one graph launch
    per solve (device-side stopping test), as one launch per block of steps
    with a host check, and launched kernel by kernel: the same iterates, so
    the same eigenpairs to the last bit."""
    n, nev, target = 4, 3, 6.0
    kvec = fame.fcc_point("X")
    out = {}
    for g in (2, 1, 0):
        plan = fame.woodpile_plan(n, [kvec], gamma=0.5)
        plan.set_option("graph", g)
        r = plan.jdsira(nev, target=target, tol=1e-8, no_restart=30, restart_dim=4, inner_tol=1e-2,
                        inner_prec="c128", want_vectors=False, shift=target)
        assert r["status"] == 0
        out[g] = (np.asarray(r["ew"]), np.asarray(r["res"]))
        plan.close()
    for g in (2, 1):
        assert np.array_equal(out[g][0], out[0][0]) and np.array_equal(out[g][1], out[0][1])
