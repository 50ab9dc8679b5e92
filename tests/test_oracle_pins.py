"""Pins of the CPU oracle.  The reference ships no golden vectors and MATLAB
cannot run here, so the oracle is pinned by the reference's own in-code
identity checks (evaluated with its explicit sparse operators) and by a
closed form for homogeneous media derived independently."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O

THETAS = [(np.pi, 0.0, np.pi), (0.3, -1.1, 2.5), (1e-4 * 0.5, 1e-4, 1e-4 * 0.5)]


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("th", THETAS)
def test_svd_1d_identities(n, th):
    # SVD_Matrix_1D.m:50-59,92: K_m = V_m Lambda U_m^H with V_m = U_m = diag(S) F_m,
    # and ifft(x)*sqrt(m) = F_m x.
    for t in th:
        K = O.K_QPBC(n, t, 1.0 / n).toarray()
        F = O.DFT_mtx(n)
        V = np.diag(O.S_sDFT(n, t)) @ F
        lam = O.lambda_quasi_periodic(n, t, 1.0 / n)
        assert np.linalg.norm(K - V @ np.diag(lam) @ V.conj().T) < 1e-11 * n
    x = np.random.default_rng(0).random(n) + 1j * np.random.default_rng(1).random(n)
    assert np.linalg.norm(np.fft.ifft(x) * np.sqrt(n) - O.DFT_mtx(n) @ x) < 1e-13


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("th", THETAS)
def test_curl_svd_identities(n, th):
    # Funhand_Generate_Lanzcos.m:176-177,213-214,218-219 against the explicit curl C.
    dims = O.Dims(n, n, n)
    svd = O.svd_matrix_generate(dims, th)
    f = O.make_handles(svd)
    C = O.curl_C(dims.shape, th, dims.mesh_len)
    rng = np.random.default_rng(7)
    N = dims.Nq
    x3 = rng.random(3 * N) + 1j * rng.random(3 * N)
    x2 = rng.random(2 * N) + 1j * rng.random(2 * N)
    scale = np.linalg.norm(C @ x3) + 1
    assert np.linalg.norm(C @ x3 - f.Psi(svd.Lambda_orig @ f.Phis(x3))) < 1e-12 * scale        # DFT_C
    assert np.linalg.norm(C.conj().T @ x3 - f.Phi(svd.Lambda_orig.conj().T @ f.Psis(x3))) < 1e-12 * scale
    assert np.linalg.norm(C @ x3 - f.Pr(svd.Sigma_r * f.Qrs(x3))) < 1e-12 * scale              # cSVD_C
    assert np.linalg.norm(C.conj().T @ x3 - f.Qr(svd.Sigma_r * f.Prs(x3))) < 1e-12 * scale     # cSVD_Cs
    assert np.linalg.norm(f.Qrs(f.Qr(x2)) - x2) < 1e-12 * np.linalg.norm(x2)                    # orth_Qr
    assert np.linalg.norm(f.Prs(f.Pr(x2)) - x2) < 1e-12 * np.linalg.norm(x2)                    # orth_Pr


@pytest.mark.parametrize("th", THETAS[:2])
def test_svd_generate_identities(th):
    # SVD_Matrix_Generate.m:59-64,74-75,99-102: per-partial SVDs, compact Lambda,
    # semi-orthogonality of Pr and Qr.
    n = 4
    dims = O.Dims(n, n, n)
    svd = O.svd_matrix_generate(dims, th)
    Vm = [np.diag(O.S_sDFT(n, t)) @ O.DFT_mtx(n) for t in th]
    Psi = np.kron(Vm[2], np.kron(Vm[1], Vm[0]))  # all Psi_c / Phi_c coincide for QP
    C = O.curl_C(dims.shape, th, dims.mesh_len).toarray()
    N = dims.Nq
    Pbig = np.kron(np.eye(3), Psi)
    assert np.linalg.norm(C @ Pbig - Pbig @ svd.Lambda_r.toarray()) < 1e-10 * np.linalg.norm(C)  # Compact_C
    Lr = svd.Lambda_r.toarray()
    Pq = np.hstack([svd.Pi0.conj().toarray(), svd.Pr.toarray()])
    Qq = np.hstack([svd.Pi0.toarray(), svd.Qr.toarray()])
    Sq = np.diag(np.concatenate([np.zeros(N), svd.Sigma_r]))
    assert np.linalg.norm(Lr - Pq @ Sq @ Qq.conj().T) < 1e-10 * np.linalg.norm(Lr)  # SVD_Lambda_r
    for M in (svd.Pr.toarray(), svd.Qr.toarray()):
        assert np.linalg.norm(M.conj().T @ M - np.eye(2 * N)) < 1e-12 * N                # semiorig


def test_material_operators_hermitian_and_pd():
    # Interpolation_Material_Matrix_Mult_Point_vertex.m:22-26 symmetrises N, M.
    P = O.build_problem(4, wave_vec=O.fcc_vertex("L"), gamma=0.2)
    for M in (P.mat.N_int, P.mat.M_int):
        assert abs(M - M.conj().T).max() < 1e-14
    big = sp.bmat([[P.mat.M_int, P.mat.J_intH], [P.mat.J_int, P.mat.N_int]]).toarray()
    w = np.linalg.eigvalsh(0.5 * (big + big.conj().T))
    assert w.min() > 0  # the material operator of a bi-isotropic woodpile is HPD


def homogeneous_eigs(n, th, blocks):
    """Closed form of the GEP  A x = lam B x  for a homogeneous medium: every
    shift is Fourier-diagonal, T_d <-> t_d = exp(i(2 pi k_d + theta_d)/n), so
    B is block diagonal with 4x4 blocks Pi^H G(k) Pi per frequency."""
    Nb, Mb, Jb = [b.reshape(3, 3) for b in blocks]
    Nh = 0.5 * (Nb + Nb.conj().T)
    Mh = 0.5 * (Mb + Mb.conj().T)
    w = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    ev = []
    for k3 in range(n):
        for k2 in range(n):
            for k1 in range(n):
                k = (k1, k2, k3)
                t = [np.exp(1j * (2 * np.pi * k[d] + th[d]) / n) for d in range(3)]
                L = np.array([(t[d] - 1.0) * n for d in range(3)])
                c = [1.0 + t[d] for d in range(3)]
                ax = lambda i: [d for d in range(3) if d != i]
                G = np.zeros((6, 6), complex)
                for i in range(3):
                    for j in range(3):
                        ki, kj = ax(i), ax(j)
                        if i == j:
                            G[i, j] = Mh[i, i].real
                            G[3 + i, 3 + j] = Nh[i, i].real
                        else:
                            G[i, j] = c[ki[0]] * c[ki[1]] * Mh[i, j] * np.conj(c[kj[0]] * c[kj[1]]) / 16
                            G[3 + i, 3 + j] = c[i] * Nh[i, j] * np.conj(c[j]) / 4
                        G[3 + i, j] = c[i] * Jb[i, j] * np.conj(c[kj[0]] * c[kj[1]]) / 8
                G[:3, 3:] = G[3:, :3].conj().T
                lq = np.sum(np.abs(L) ** 2)
                p1 = np.cross(np.conj(L), w)
                p1 = p1 / np.linalg.norm(p1)
                p2 = np.cross(np.conj(p1), np.conj(L)) / np.sqrt(lq)
                Pi = np.zeros((6, 4), complex)
                Pi[:3, 0], Pi[:3, 1] = -np.conj(p2), np.conj(p1)
                Pi[3:, 2], Pi[3:, 3] = p1, p2
                Bk = Pi.conj().T @ G @ Pi
                s = 1.0 / np.sqrt(lq)
                Ak = np.zeros((4, 4), complex)
                Ak[0, 2] = Ak[1, 3] = 1j * s
                Ak[2, 0] = Ak[3, 1] = -1j * s
                Lc = np.linalg.cholesky(0.5 * (Bk + Bk.conj().T))
                Li = np.linalg.inv(Lc)
                ev.extend(np.linalg.eigvalsh(Li @ Ak @ Li.conj().T))
    return np.sort(np.array(ev))[::-1]


@pytest.mark.parametrize("gamma", [0.0, 0.3])
def test_homogeneous_closed_form_lanczos(gamma):
    n = 4
    th = (0.7, -0.4, 1.3)
    ph = O.woodpile_phases(gamma, eps_in=3.0)
    A = O.fcc_lattice()
    blocks = O.material_blocks(ph[1], A)
    inside = np.ones(n ** 3, dtype=bool)  # the whole cell is the rod material
    P = O.build_problem(n, thetas=th, inside=inside, phases=ph)
    k = 6
    ref = homogeneous_eigs(n, th, [b.ravel() for b in blocks])[:k]
    L = 4 * n ** 3
    ev, ew, it = O.lanczos(P.A, P.B, lambda r: O.fncinvB(r, P.B, 1e-13, 10000), L, k, 1e-12, 200, 2 * k,
                           np.ones(L, complex))
    assert np.allclose(ew, ref, rtol=1e-9, atol=0)


def test_lanczos_residuals_small():
    # EvaluteError_Chiral_no_inv.m:18-20: NFSEP and ORGSEP residuals of converged pairs
    n = 4
    P = O.build_problem(n, wave_vec=O.fcc_vertex("X"), gamma=0.2)
    L = 4 * n ** 3
    k = 4
    ev, ew, it = O.lanczos(P.A, P.B, lambda r: O.fncinvB(r, P.B, 1e-12, 10000), L, k, 1e-10, 100, 2 * k,
                           np.ones(L, complex))
    omega = 1.0 / ew
    E, H = O.eigen_restoration(ev, P.fnc, P.mat)
    rn, ro = O.evaluate_error(ev, omega, E, H, P.dims, P.thetas, P.A, P.B, P.mat)
    assert np.all(rn < 1e-8)
    assert np.all(ro < 1e-7 * np.max(np.abs(omega)) * n)
