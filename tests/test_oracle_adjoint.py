"""The oracle's eigenfrequency gradient with respect to per-vertex chiral
fields (field_gradient: Hellmann-Feynman through the literal sparse assembly)
against central finite differences of dense FP64 eigenvalues.

A per-voxel difference quotient with step 1e-6 needs eigenvalues accurate to
far below 1e-12 relative, which only a dense solve gives, so the check runs
at n = 4 (256 unknowns): the objective is the gap between bands 2 and 3
summed over k-points on the Gamma-X-W-L path; 32 seeded voxels per field.
Gamma itself is left out of the difference quotients: with the +1e-4 shift
||fncA|| ~ 1/sigma_min ~ 1e4, so dense eigenvalues there carry absolute
errors near 1e-11, larger than what a 1e-6 step resolves."""
import numpy as np
import pytest
import scipy.linalg as sla

import oracle as O

N = 4


def dense_solver(n, thetas):
    """Dense B(eps, gamma) = Y^H K Y with Y = blkdiag(Pr, Qr) built once."""
    eps0 = np.full(n ** 3, 2.0)
    P = O.build_problem_field(n, eps0, np.zeros(n ** 3), thetas=thetas)
    Nq = n ** 3
    I2 = np.eye(2 * Nq, dtype=complex)
    Yu = np.stack([P.fnc.Pr(I2[:, j]) for j in range(2 * Nq)], axis=1)
    Yv = np.stack([P.fnc.Qr(I2[:, j]) for j in range(2 * Nq)], axis=1)
    L4 = np.eye(4 * Nq, dtype=complex)
    A = np.stack([P.A(L4[:, j]) for j in range(4 * Nq)], axis=1)
    A = 0.5 * (A + A.conj().T)

    def omegas(eps, gam):
        (Nv, Mv, Jv), _ = O.field_diagonals(eps, gam)
        Nint, Mint, Jint = O.interp_material_vertex(P.dims, thetas, Nv, Mv, Jv)
        uu = Yu.conj().T @ (Mint @ Yu)
        vv = Yv.conj().T @ (Nint @ Yv)
        vu = Yv.conj().T @ (Jint @ Yu)
        B = np.block([[uu, vu.conj().T], [vu, vv]])
        B = 0.5 * (B + B.conj().T)
        mu, X = sla.eigh(A, B)
        om = 1.0 / mu
        pos = np.where(om > 0)[0]
        order = pos[np.argsort(om[pos])]
        return om[order], X[:, order]

    return omegas


@pytest.fixture(scope="module", autouse=True)
def one_blas_thread():
    """256x256 solves run fastest single-threaded."""
    try:
        from threadpoolctl import threadpool_limits
    except ImportError:
        yield
        return
    with threadpool_limits(1):
        yield


@pytest.fixture(scope="module")
def setup():
    A = O.fcc_lattice()
    G, X = O.fcc_vertex("G", A), O.fcc_vertex("X", A)
    kpts = [0.5 * (G + X)] + [O.fcc_vertex(lab, A) for lab in ("X", "W", "L")]
    ths = [O.thetas_from_k(k, A) for k in kpts]
    eps, gam = O.chiral_noise_field(N, seed=5, sigma=1.0)
    return ths, eps, gam, [dense_solver(N, th) for th in ths]


def gap(solvers, eps, gam):
    tot = 0.0
    for s in solvers:
        om, _ = s(eps, gam)
        tot += om[2] - om[1]
    return tot


def analytic(ths, solvers, eps, gam):
    ge = np.zeros(N ** 3)
    gg = np.zeros(N ** 3)
    for th, s in zip(ths, solvers):
        om, X = s(eps, gam)
        P = O.build_problem_field(N, eps, gam, thetas=th)
        for b, w in ((2, 1.0), (1, -1.0)):
            assert abs(om[b] - om[b - 1]) > 1e-6 * om[b] and abs(om[b + 1] - om[b]) > 1e-6 * om[b]
            e_, g_, xbx = O.field_gradient(P, X[:, b], om[b], eps, gam)
            assert abs(xbx - 1.0) < 1e-10  # eigh returns B-normalised vectors
            ge += w * e_
            gg += w * g_
    return ge, gg


@pytest.mark.parametrize("which", ["eps", "gamma"])
def test_gradient_matches_central_differences(setup, which):
    ths, eps, gam, solvers = setup
    ge, gg = analytic(ths, solvers, eps, gam)
    g = ge if which == "eps" else gg
    rng = np.random.default_rng(7)
    vox = rng.choice(N ** 3, 32, replace=False)
    h = 1e-6
    for v in vox:
        e1, e2, g1, g2 = eps.copy(), eps.copy(), gam.copy(), gam.copy()
        if which == "eps":
            e1[v] += h
            e2[v] -= h
        else:
            g1[v] += h
            g2[v] -= h
        fd = (gap(solvers, e1, g1) - gap(solvers, e2, g2)) / (2 * h)
        # relative 1e-5, plus the quotient's rounding floor: eight eigenvalues
        # near 0.7 each rounded to ~1e-16, divided by 2h
        assert abs(fd - g[v]) <= 1e-5 * abs(g[v]) + 2e-9, (v, fd, g[v])


def test_quadratic_form_is_xBx(setup):
    ths, eps, gam, _ = setup
    P = O.build_problem_field(N, eps, gam, thetas=ths[1])
    rng = np.random.default_rng(1)
    x = rng.standard_normal(4 * N ** 3) + 1j * rng.standard_normal(4 * N ** 3)
    _, _, xbx = O.field_gradient(P, x, 1.0, eps, gam)
    assert abs(xbx - np.vdot(x, P.B(x)).real) <= 1e-12 * abs(xbx)
