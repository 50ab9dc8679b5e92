"""FP64 CPU restatement of the reference's quasi-periodic FFT eigensolver path.

TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
product library never imports this module.

Every function follows a file of the reference (FAME-GPU/3D-Bi-Anisotropic-PhC)
and cites it as ``path:line``.  Vectors use the reference's MATLAB ordering:
column-major grids (x fastest), components stacked 1, 2, 3.  Only
quasi-periodic ('QP') boundary conditions are restated: every configuration
of the reference's band-structure and light-localisation scripts uses them
(``InputData/BS_Gyroid/Physical_settings_woodpile.m:100-105``), and the
DCT/DST branches are dead code on that path.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft
import scipy.sparse as sp

__all__ = [
    "distop_theta", "lambda_quasi_periodic", "S_sDFT", "K_QPBC", "DFT_mtx",
    "curl_C", "Dims", "SVDData", "svd_matrix_generate", "mtxvecmul_fft",
    "Handles", "make_handles", "fcc_lattice", "reciprocal", "fcc_vertex",
    "thetas_from_k", "grid_vertices", "woodpile_isofun", "sphere_isofun",
    "tetra_isofun", "Phase", "material_blocks", "dist_material",
    "interp_material_vertex", "MaterialOps", "fncA", "fncB", "pcg_matlab",
    "fncinvB", "lanczos", "eigen_restoration", "evaluate_error",
    "BandProblem", "build_problem", "woodpile_phases", "fft_workers",
    "field_diagonals", "build_problem_field", "material_quad_coeffs", "field_gradient",
    "chiral_noise_field", "lanczos_gep", "gsreorthog",
    "gram_schmidt_ref", "choose_ritz_pair_cl", "sira_correction", "jdsira_driver4",
]

_W = max(1, min(8, os.cpu_count() or 1))


def fft_workers(n: int | None = None) -> int:
    """Threads handed to ``scipy.fft`` (all host cores, at most 8 by default)."""
    global _W
    if n is not None:
        _W = max(1, int(n))
    return _W


# --------------------------------------------------------------------------
# @DistOp: 1D symbols and operators
# --------------------------------------------------------------------------
def distop_theta(m, k):
    """``@DistOp/theta.m:2``: ``(k-1)*pi/m``."""
    return (np.asarray(k, dtype=np.float64) - 1.0) * np.pi / m


def lambda_quasi_periodic(m, theta, delta):
    """``@DistOp/lambda_QuasiPeriodic.m:3``: singular values of ``K_QPBC``."""
    j = np.arange(1, m + 1)
    return (np.exp(1j * (2.0 * distop_theta(m, j) + theta / m)) - 1.0) / delta


def S_sDFT(m, theta):
    """``@DistOp/S_sDFT.m:2``: the Bloch phase ``exp(1i*(0:m-1)'*theta/m)``."""
    return np.exp(1j * np.arange(m) * theta / m)


def K_QPBC(m, theta, delta):
    """``@DistOp/K_QPBC.m:3``: forward difference with quasi-periodic wrap."""
    rows = np.r_[np.arange(m), np.arange(m)]
    cols = np.r_[np.arange(m), np.arange(1, m), 0]
    vals = np.r_[-np.ones(m), np.ones(m - 1), np.exp(1j * theta)].astype(np.complex128)
    return sp.csr_matrix((vals, (rows, cols)), shape=(m, m)) / delta


def DFT_mtx(m):
    """``@DistOp/DFT_mtx.m:3``: unitary m-by-m (inverse-sign) DFT matrix."""
    j = np.arange(m)[:, None]
    return np.sqrt(1.0 / m) * np.exp(2j * j * distop_theta(m, np.arange(1, m + 1))[None, :])


def _I(m):
    return sp.identity(m, dtype=np.complex128, format="csr")


def curl_C(dims, thetas, delta):
    """``@DistOp/C.m:3-5`` with ``C_12 .. C_32`` (QP: row = col = n).

    ``C = [0 -C13 C12; C23 0 -C21; -C32 C31 0]`` where ``C_ij`` is the
    forward difference along axis ``j`` (``@DistOp/C_12.m:2`` etc.).
    """
    n1, n2, n3 = dims
    Kx = K_QPBC(n1, thetas[0], delta[0])
    Ky = K_QPBC(n2, thetas[1], delta[1])
    Kz = K_QPBC(n3, thetas[2], delta[2])
    C12 = sp.kron(_I(n3), sp.kron(Ky, _I(n1)))
    C13 = sp.kron(Kz, sp.kron(_I(n2), _I(n1)))
    C21 = sp.kron(_I(n3), sp.kron(_I(n2), Kx))
    C23 = sp.kron(Kz, sp.kron(_I(n2), _I(n1)))
    C31 = sp.kron(_I(n3), sp.kron(_I(n2), Kx))
    C32 = sp.kron(_I(n3), sp.kron(Ky, _I(n1)))
    N = n1 * n2 * n3
    O = sp.csr_matrix((N, N), dtype=np.complex128)
    return sp.bmat([[O, -C13, C12], [C23, O, -C21], [-C32, C31, O]], format="csr")


def shift_diff(dims, thetas, axis):
    """``@DistOp/C_b1.m:2`` (and ``C_b2``, ``C_b3``) with ``delta = 1``.

    ``I + C_b{d}`` is the Bloch forward shift along axis ``d``.
    """
    n1, n2, n3 = dims.shape if isinstance(dims, Dims) else dims
    if axis == 0:
        return sp.kron(_I(n3), sp.kron(_I(n2), K_QPBC(n1, thetas[0], 1.0))).tocsr()
    if axis == 1:
        return sp.kron(_I(n3), sp.kron(K_QPBC(n2, thetas[1], 1.0), _I(n1))).tocsr()
    return sp.kron(K_QPBC(n3, thetas[2], 1.0), sp.kron(_I(n2), _I(n1))).tocsr()


# --------------------------------------------------------------------------
# SVD of the discrete curl (QP)
# --------------------------------------------------------------------------
@dataclass
class Dims:
    """``InputData/BS_Gyroid/Computational_settings_Lanczos.m:37-101`` for QP."""
    n1: int
    n2: int
    n3: int

    @property
    def shape(self):
        return (self.n1, self.n2, self.n3)

    @property
    def Nq(self):
        return self.n1 * self.n2 * self.n3

    @property
    def mesh_len(self):
        # lattice constant 1: Computational_settings_Lanczos.m:38
        return (1.0 / self.n1, 1.0 / self.n2, 1.0 / self.n3)


@dataclass
class SVDData:
    dims: Dims
    thetas: tuple
    lam1d: list            # [lx, ly, lz]
    Lx: np.ndarray
    Ly: np.ndarray
    Lz: np.ndarray
    Lambda_q: np.ndarray
    Sigma_r: np.ndarray    # 2Nq
    Pi0: sp.csr_matrix
    Pi1: sp.csr_matrix
    Pi2: sp.csr_matrix
    Pr: sp.csr_matrix      # 3Nq x 2Nq
    Qr: sp.csr_matrix      # 3Nq x 2Nq
    S: np.ndarray          # 3Nq Bloch phase (Psi and Phi coincide for QP)
    D: np.ndarray          # 3Nq, ones for QP
    Lambda_orig: sp.csr_matrix = None
    Lambda_r: sp.csr_matrix = None


def svd_matrix_generate(dims: Dims, thetas) -> SVDData:
    """QP branch of ``subroutines/SVD_Matrix_Generate.m:24-30``.

    1D symbols: ``SVD_Matrix_1D.m:29-48``; 3D diagonals: ``SVD_Matrix_3D.m:8-17``;
    phases ``S``: ``SVD_Matrix_3D.m:79-86``; curl SVD blocks:
    ``SVD_Matrix_curl.m:23-89`` (with ``Ntil = 0`` for QP).
    """
    n1, n2, n3 = dims.shape
    hx, hy, hz = dims.mesh_len
    lx = lambda_quasi_periodic(n1, thetas[0], hx)
    ly = lambda_quasi_periodic(n2, thetas[1], hy)
    lz = lambda_quasi_periodic(n3, thetas[2], hz)
    N = dims.Nq
    Dx, Dy, Dz = sp.diags(lx), sp.diags(ly), sp.diags(lz)
    # SVD_Matrix_3D.m:8-13
    C13 = sp.kron(Dz, sp.kron(_I(n2), _I(n1)))
    C12 = sp.kron(_I(n3), sp.kron(Dy, _I(n1)))
    C23 = sp.kron(Dz, sp.kron(_I(n2), _I(n1)))
    C21 = sp.kron(_I(n3), sp.kron(_I(n2), Dx))
    C32 = sp.kron(_I(n3), sp.kron(Dy, _I(n1)))
    C31 = sp.kron(_I(n3), sp.kron(_I(n2), Dx))
    # SVD_Matrix_3D.m:15-17
    L3x = sp.kron(_I(n3), sp.kron(_I(n2), Dx)).tocsr()
    L3y = sp.kron(_I(n3), sp.kron(Dy, _I(n1))).tocsr()
    L3z = sp.kron(Dz, sp.kron(_I(n2), _I(n1))).tocsr()
    O = sp.csr_matrix((N, N), dtype=np.complex128)
    # SVD_Matrix_curl.m:23-32
    Lambda_orig = sp.bmat([[O, -C13, C12], [C23, O, -C21], [-C32, C31, O]], format="csr")
    Lambda_r = sp.bmat([[O, -L3z, L3y], [L3z, O, -L3x], [-L3y, L3x, O]], format="csr")
    # SVD_Matrix_curl.m:45-57
    w = np.arange(1, 4, dtype=np.float64)
    w = w / np.linalg.norm(w)
    Lambda_q = (L3x.conj().T @ L3x + L3y.conj().T @ L3y + L3z.conj().T @ L3z)
    Lambda_w = w[0] * L3x + w[1] * L3y + w[2] * L3z
    norm_Pi_0 = np.sqrt(Lambda_q.diagonal())
    inv_norm_Pi_0 = sp.diags(1.0 / norm_Pi_0)
    norm_Pi_1 = np.sqrt((Lambda_q - Lambda_w.conj().T @ Lambda_w).diagonal())
    inv_norm_Pi_1 = sp.diags(1.0 / norm_Pi_1)
    Pi0 = (sp.vstack([L3x, L3y, L3z]) @ inv_norm_Pi_0).tocsr()
    kron_w = sp.kron(sp.csr_matrix(w.reshape(3, 1)), _I(N))
    Pi1 = (-Lambda_r.conj().T @ kron_w @ inv_norm_Pi_1).tocsr()
    Pi2 = (Lambda_r.conj().T @ Pi1.conj() @ inv_norm_Pi_0).tocsr()
    # SVD_Matrix_curl.m:63-64,67,74,88-89 (I.Psi = I.Phi = I, Ntil = 0)
    Qr = sp.hstack([Pi1, Pi2], format="csr")
    Pr = sp.hstack([-Pi2.conj(), Pi1.conj()], format="csr")
    sqrt_lq = np.sqrt(Lambda_q.diagonal().real)
    Sigma_r = np.concatenate([sqrt_lq, sqrt_lq])
    # SVD_Matrix_3D.m:79-86 with SVD_Matrix_1D.m:37,45 (U.S = V.S)
    Sx, Sy, Sz = S_sDFT(n1, thetas[0]), S_sDFT(n2, thetas[1]), S_sDFT(n3, thetas[2])
    S1 = np.kron(Sz, np.kron(Sy, Sx))
    S = np.concatenate([S1, S1, S1])
    D = np.ones(3 * N, dtype=np.complex128)  # @DistOp/D_sDFT.m
    return SVDData(dims, tuple(thetas), [lx, ly, lz], L3x.diagonal(), L3y.diagonal(),
                   L3z.diagonal(), Lambda_q.diagonal().real, Sigma_r, Pi0, Pi1, Pi2,
                   Pr, Qr, S, D, Lambda_orig, Lambda_r)


def mtxvecmul_fft(vec_in, dims: Dims, istrans: str, S, D):
    """``subroutines/MtxVecMul_FFT.m:18-62`` for 'DFT' types (P, R identities).

    'notranspose': ``S .* [ifftn(Y_c)*sqrt(N)]``; 'transpose': the adjoint
    ``conj(D) .* [fftn(conj(S).*Y_c)/sqrt(N)]``.
    """
    n1, n2, n3 = dims.shape
    N = dims.Nq
    norm_c = math.sqrt(N)
    vec_in = np.asarray(vec_in)
    out = np.empty(3 * N, dtype=np.complex128)
    if istrans == "notranspose":
        x = D * vec_in
        for c in range(3):
            Y = x[c * N:(c + 1) * N].reshape((n1, n2, n3), order="F")
            Y = sfft.ifftn(Y, workers=_W) * norm_c
            out[c * N:(c + 1) * N] = Y.reshape(-1, order="F")
        return S * out
    if istrans == "transpose":
        x = np.conj(S) * vec_in
        for c in range(3):
            Y = x[c * N:(c + 1) * N].reshape((n1, n2, n3), order="F")
            Y = sfft.fftn(Y, workers=_W) / norm_c
            out[c * N:(c + 1) * N] = Y.reshape(-1, order="F")
        return np.conj(D) * out
    raise ValueError("istrans must be 'notranspose' or 'transpose'")


@dataclass
class Handles:
    """``fun_Lanczos/Funhand_Generate_Lanzcos.m:36-41,79-82`` (GPU branch).

    For QP boundaries ``Psi`` and ``Phi`` share ``S``, ``D`` and sizes.
    """
    svd: SVDData

    def Psi(self, x):
        return mtxvecmul_fft(x, self.svd.dims, "notranspose", self.svd.S, self.svd.D)

    Phi = Psi

    def Psis(self, x):
        return mtxvecmul_fft(x, self.svd.dims, "transpose", self.svd.S, self.svd.D)

    Phis = Psis

    def Pr(self, x):   # Funhand_Generate_Lanzcos.m:79
        return self.Psi(self.svd.Pr @ x)

    def Qr(self, x):   # :80
        return self.Phi(self.svd.Qr @ x)

    def Prs(self, x):  # :81
        return self.svd.Pr.conj().T @ self.Psis(x)

    def Qrs(self, x):  # :82
        return self.svd.Qr.conj().T @ self.Phis(x)


def make_handles(svd: SVDData) -> Handles:
    return Handles(svd)


# --------------------------------------------------------------------------
# Lattice, geometry and material
# --------------------------------------------------------------------------
def fcc_lattice(a=1.0):
    """``Physical_settings_woodpile.m:7``: columns are the primitive vectors."""
    return 0.5 * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], dtype=np.float64) * a


def reciprocal(A):
    """``Physical_settings_woodpile.m:9``: ``2*pi*inv(A')``."""
    return 2.0 * np.pi * np.linalg.inv(A.T)


def fcc_vertex(name, A=None):
    """FCC high-symmetry points, ``Physical_settings_woodpile.m:143-148``."""
    A = fcc_lattice() if A is None else A
    B = reciprocal(A)
    tab = {"G": (0, 0, 0), "K": (3 / 8, 3 / 8, 3 / 4), "L": (0.5, 0.5, 0.5),
           "U": (5 / 8, 1 / 4, 5 / 8), "W": (0.5, 1 / 4, 3 / 4), "X": (0.5, 0, 0.5)}
    return B @ np.array(tab[name], dtype=np.float64)


def thetas_from_k(wave_vec, A=None):
    """``band_structure_woodpile_Lanczos_n60_gamma0p2.m:50-56``.

    A zero wave vector is shifted by 1e-4 in every component before the Bloch
    angles ``theta_d = k . a_d`` are formed.
    """
    A = fcc_lattice() if A is None else A
    k = np.asarray(wave_vec, dtype=np.float64).copy()
    if np.linalg.norm(k) == 0:
        k = k + 1e-4
    return tuple(float(np.dot(k, A[:, d])) for d in range(3))


def grid_vertices(dims: Dims):
    """``Public/Grid_Generate_Mult_Point.m:7-17``: vertex lattice coefficients."""
    n1, n2, n3 = dims.shape
    r1 = np.arange(n1) / n1
    r2 = np.arange(n2) / n2
    r3 = np.arange(n3) / n3
    coef = np.empty((dims.Nq, 3))
    coef[:, 0] = np.kron(np.ones(n3 * n2), r1)
    coef[:, 1] = np.kron(np.ones(n3), np.kron(r2, np.ones(n1)))
    coef[:, 2] = np.kron(r3, np.ones(n2 * n1))
    return coef


def woodpile_isofun(P, w, a):
    """``Public/woodpile_isofun.m:1-13`` (returns a boolean mask)."""
    x, y, z = P[:, 0], P[:, 1], P[:, 2]
    t1 = y - x
    t2 = y + x
    w = math.sqrt(2) / 2 * w
    m = (((z >= 0) & (z < a / 4)) & ((t1 >= (a - w)) | (t1 <= -(a - w)) | ((t1 >= -w) & (t1 <= w)))) \
        | (((z >= a / 4) & (z < a / 2)) & (((t2 >= 3 * a / 2 - w) & (t2 <= 3 * a / 2 + w))
                                          | ((t2 >= a / 2 - w) & (t2 <= a / 2 + w)))) \
        | (((z >= a / 2) & (z < 3 * a / 4)) & (((t1 >= (-a / 2 - w)) & (t1 <= (-a / 2 + w)))
                                              | ((t1 >= (a / 2 - w)) & (t1 <= (a / 2 + w))))) \
        | (((z >= 3 * a / 4) & (z <= a)) & ((t2 >= (2 * a - w)) | (t2 <= w) | ((t2 >= a - w) & (t2 <= a + w))))
    return m


def sphere_isofun(P, centers, radius):
    """``Physical_settings_sphere``-style inclusion (``Physical_settings_woodpile.m:18,32``):
    inside when ``-min_c |r - c| > -radius``."""
    centers = np.atleast_2d(centers)
    d = np.min(np.linalg.norm(P[:, None, :] - centers[None, :, :], axis=2), axis=1)
    return -d > -radius


def tetra_isofun(P, verts):
    """Regular tetrahedron inclusion by four same-side-of-plane tests, as in
    ``subroutines/Material_Locate_Isofunction.m:38-90,135-148`` (case 1 with
    a degenerate apex set): a point is inside when, for each face, it lies on
    the same side as the opposite vertex, points within 1e-8 of a plane count
    as inside."""
    verts = np.asarray(verts, dtype=np.float64)
    inside = np.ones(P.shape[0], dtype=bool)
    tol = 1e-8
    for f in range(4):
        a, b, c = [verts[i] for i in range(4) if i != f]
        q = verts[f]
        normal = np.cross(b - a, c - a)
        dp = (a - P) @ normal
        dq = np.dot(a - q, normal)
        ok = (np.abs(dp) < tol) | (abs(dq) < tol) | (dp * dq > 0)
        inside &= ok
    return inside


@dataclass
class Phase:
    """A homogeneous constitutive 6x6 block ``[eps xi; zeta mu]``."""
    eps: np.ndarray
    mu: np.ndarray
    xi: np.ndarray
    zeta: np.ndarray


def material_blocks(ph: Phase, A):
    """``Physical_settings_woodpile.m:91-96,184-194``: invert the 6x6 block,
    split it, and take the covariant forms ``A' X A``.

    Returns ``(N_cov, M_cov, J_cov)``: the covariant (1,1), (2,2) and (1,2)
    blocks of the inverse, which ``Material_Matrix_Generate_Mult_Point.m:28-31``
    places as ``mtx_B.N``, ``mtx_B.M`` and ``mtx_B.J``.
    """
    big = np.block([[ph.eps, ph.xi], [ph.zeta, ph.mu]]).astype(np.complex128)
    inv = np.linalg.inv(big)
    e, x, m = inv[:3, :3], inv[:3, 3:], inv[3:, 3:]
    return A.T @ (e @ A), A.T @ (m @ A), A.T @ (x @ A)


def dist_material(inside: np.ndarray, par_out: np.ndarray, par_in: np.ndarray):
    """``Material_Matrix_Generate_Mult_Point.m:38-48``: per-vertex diagonals
    ``A{i,j} = (par2(i,j)-par1(i,j))*I_tilde + par1(i,j)``."""
    I_t = inside.astype(np.float64)
    return [[(par_in[i, j] - par_out[i, j]) * I_t + par_out[i, j] for j in range(3)] for i in range(3)]


def _sd(v):
    return sp.diags(np.asarray(v, dtype=np.complex128)).tocsr()


def interp_material_vertex(dims: Dims, thetas, Nv, Mv, Jv):
    """``fun_no_inv/Interpolation_Material_Matrix_Mult_Point_vertex.m:14-27``
    with ``IntCovarFormN_vertex.m:3-14``, ``IntCovarFormM_vertex_new.m:3-19``
    and ``IntCovarFormJ_vertex_new.m:3-11``, assembled literally as sparse
    products.  ``Nv``, ``Mv``, ``Jv`` are 3x3 nested lists of per-vertex
    diagonals.  ``N_int`` and ``M_int`` are symmetrised ``(X+X')/2``; ``J_int``
    is not.
    """
    N = dims.Nq
    I = _I(N)
    C = [shift_diff(dims, thetas, d) for d in range(3)]
    CH = [c.conj().T.tocsr() for c in C]

    def k_of(i):
        return [d for d in range(3) if d != i]

    # IntCovarFormN_vertex (P = I_R1 = identity for QP)
    tN = [[None] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(3):
            A = _sd(Nv[i][j])
            if i != j:
                tN[i][j] = 0.25 * (2 * I + C[i]) @ A @ (2 * I + CH[j])
            else:
                tN[i][j] = 0.5 * (A + (I + C[i]) @ A @ (I + CH[i]))
    Nint = sp.bmat(tN, format="csr")
    Nint = 0.5 * (Nint + Nint.conj().T)
    # IntCovarFormM_vertex_new
    tM = [[None] * 3 for _ in range(3)]
    for i in range(3):
        k = k_of(i)
        for j in range(3):
            A = _sd(Mv[i][j])
            if i == j:
                t1, t2 = (I + C[k[0]]), (I + C[k[1]])
                tM[i][i] = 0.25 * (A + t1 @ A @ t1.conj().T + t2 @ A @ t2.conj().T
                                   + t1 @ t2 @ A @ t2.conj().T @ t1.conj().T)
            else:
                l = k_of(j)
                tM[i][j] = (1.0 / 16) * (2 * I + C[k[0]]) @ (2 * I + C[k[1]]) @ A \
                    @ (2 * I + CH[l[1]]) @ (2 * I + CH[l[0]])
    Mint = sp.bmat(tM, format="csr")
    Mint = 0.5 * (Mint + Mint.conj().T)
    # IntCovarFormJ_vertex_new
    tJ = [[None] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(3):
            k = k_of(j)
            A = _sd(Jv[i][j])
            tJ[i][j] = 0.125 * (2 * I + C[i]) @ A @ (2 * I + CH[k[1]]) @ (2 * I + CH[k[0]])
    Jint = sp.bmat(tJ, format="csr")
    return Nint.tocsr(), Mint.tocsr(), Jint.tocsr()


@dataclass
class MaterialOps:
    N_int: sp.csr_matrix
    M_int: sp.csr_matrix
    J_int: sp.csr_matrix
    J_intH: sp.csr_matrix = None

    def __post_init__(self):
        if self.J_intH is None:
            self.J_intH = self.J_int.conj().T.tocsr()


# --------------------------------------------------------------------------
# Operator handles
# --------------------------------------------------------------------------
def fncA(x, Sigma_r):
    """``fun_Lanczos/fncA.m:3-4``: ``[1i*inv_r.*x2; -1i*inv_r.*x1]``."""
    inv_r = 1.0 / Sigma_r
    h = x.shape[0] // 2
    return np.concatenate([1j * inv_r * x[h:], -1j * inv_r * x[:h]])


def fncB(x, fnc: Handles, mat: MaterialOps):
    """``fun_Lanczos/fncB.m:3-6`` (= ``fun_no_inv/fncB_Generate_no_inv.m:6-8``)."""
    h = x.shape[0] // 2
    u = fnc.Pr(x[:h])
    v = fnc.Qr(x[h:])
    up = mat.M_int @ u + mat.J_intH @ v
    vp = mat.J_int @ u + mat.N_int @ v
    return np.concatenate([fnc.Prs(up), fnc.Qrs(vp)])


def pcg_matlab(op, b, tol, maxit, x0=None):
    """Unpreconditioned conjugate gradients with MATLAB ``pcg``'s stopping rule
    ``norm(b - A*x) <= tol*norm(b)`` (used by ``fun_Lanczos/fncinvB.m:4``).

    Returns ``(x, flag, relres, iters)``; flag 0 means converged.
    """
    x = np.zeros_like(b) if x0 is None else x0.copy()
    nb = np.linalg.norm(b)
    if nb == 0:
        return np.zeros_like(b), 0, 0.0, 0
    r = b - op(x) if x0 is not None else b.copy()
    p = r.copy()
    rho = np.vdot(r, r).real
    for it in range(1, maxit + 1):
        q = op(p)
        alpha = rho / np.vdot(p, q).real
        x += alpha * p
        r -= alpha * q
        rho_new = np.vdot(r, r).real
        if math.sqrt(rho_new) <= tol * nb:
            return x, 0, math.sqrt(rho_new) / nb, it
        p = r + (rho_new / rho) * p
        rho = rho_new
    return x, 1, math.sqrt(rho) / nb, maxit


def fncinvB(x, B_op, tol=1e-12, maxit=10000, stats=None):
    """``fun_Lanczos/fncinvB.m:4``: ``pcg(B_op, x, tol, maxit)``, flag ignored."""
    y, flag, relres, it = pcg_matlab(B_op, x, tol, maxit)
    if stats is not None:
        stats.append(it)
    return y


# --------------------------------------------------------------------------
# Lanczos (Krylov-Schur) band solver
# --------------------------------------------------------------------------
def lanczos(fA, fB, fBinv, n, k, tol, maxiter, p, v0):
    """``fun_Lanczos/Lanczos.m:1-167`` line by line (CPU branch).

    Returns ``(ev, ew, iters)`` with ``ew`` the ``k`` largest eigenvalues of
    ``B^{-1}A`` (descending) and ``ev`` their B-normalised Ritz vectors.
    ``beta`` is taken as the real square root of ``r'*B*r``; MATLAB's complex
    ``sqrt`` adds an imaginary part at rounding level only.
    """
    v0 = v0 / math.sqrt(abs(np.vdot(v0, fB(v0))))                    # :8
    eps = 2.2204e-16                                                    # :23
    Q = np.zeros((n, p), dtype=np.complex128)                           # :26
    k0 = k
    Alpha, Beta = [], []
    beta = 0.0
    d = np.zeros(0)
    c = np.zeros(0)
    justRestarted = False
    sizeV = 1
    kk = 0
    v = v0
    U = None
    ind = None
    for mm in range(1, maxiter + 1):                                   # :44
        for jj in range(sizeV, p + 1):                                  # :47
            j = jj - 1
            Q[:, j] = v
            r = fA(Q[:, j])
            alpha = float(np.real(np.vdot(r, Q[:, j])))                # :51
            if jj == 1:
                pr = fBinv(r)
                r = pr - alpha * Q[:, j]
            elif justRestarted:
                pr = fBinv(r)
                r = _gs_gep(Q, pr, fB, jj)
                justRestarted = False
            else:
                pr = fBinv(r)
                r = pr - alpha * Q[:, j] - beta * Q[:, j - 1]
                r = r - np.vdot(fB(Q[:, j - 1]), r) * Q[:, j - 1]       # :63
            r = r - np.vdot(fB(Q[:, j]), r) * Q[:, j]                   # :66
            r = _gs_gep(Q, r, fB, jj)                                   # :69
            rr = fB(r)                                                  # :72
            beta = math.sqrt(abs(np.vdot(r, rr).real))                  # :73
            v = r / beta
            Alpha.append(alpha)
            Beta.append(beta)
            kk += 1
        # :93-98
        m1 = len(Alpha)
        H1 = np.diag(Alpha) + np.diag(Beta[:-1], 1) + np.diag(Beta[:-1], -1)
        kd = len(d)
        H = np.zeros((kd + m1, kd + m1))
        H[:kd, :kd] = np.diag(d)
        H[kd:, kd:] = H1
        if kd:
            H[:kd, kd] = c
            H[kd, :kd] = c
        Alpha, Beta = [], []
        dd, U = np.linalg.eigh(H)                                       # :103
        res = np.abs(beta * U[-1, :])                                   # :106
        ind = np.argsort(-dd, kind="stable")                            # :109
        dd = dd[ind]
        res = res[ind]
        isNotConverged = ~(res[:k0] < tol * np.maximum(eps ** (2.0 / 3.0), np.abs(dd[:k0])))
        nconv = int(np.count_nonzero(~isNotConverged))
        d = dd
        if nconv >= k0 or mm == maxiter:                                # :117
            break
        k = k0 + min(nconv, (p - k0) // 2)                              # :122
        if k == 1 and p > 3:
            k = p // 2
        ind = ind[:k]                                                   # :130
        Uk = U[:, ind]
        Q[:, :k] = Q @ Uk                                               # :137
        d = d[:k]
        c = beta * Uk[-1, :]                                            # :140
        justRestarted = True
        sizeV = k + 1
    Uk0 = U[:, ind[:k0]]                                                # :146
    ew = d[:k0]
    ev = Q @ Uk0                                                        # :152
    return ev, ew, kk


def _gs_gep(V, r, fB, jj):
    """``fun_Lanczos/Lanczos.m:159-167``: modified Gram-Schmidt in the B product."""
    for kq in range(jj):
        tmp = np.vdot(fB(V[:, kq]), r)
        r = r - tmp * V[:, kq]
    return r


# --------------------------------------------------------------------------
# Restoration and residuals
# --------------------------------------------------------------------------
def eigen_restoration(EV, fnc: Handles, mat: MaterialOps):
    """``fun_no_inv/Eigen_Restoration_Chiral_no_inv.m:3-25``: per column,
    ``[e;h] = -1i*[N J; J' M]*[Qr(x2); Pr(x1)]``.  Returns ``(E, H)`` with one
    column per eigenvector (each 3Nq long)."""
    E, Hs = [], []
    for j in range(EV.shape[1]):
        v = EV[:, j]
        h2 = v.shape[0] // 2
        y1 = fnc.Qr(v[h2:])
        y2 = fnc.Pr(v[:h2])
        e = -1j * (mat.N_int @ y1 + mat.J_int @ y2)
        h = -1j * (mat.J_intH @ y1 + mat.M_int @ y2)
        E.append(e)
        Hs.append(h)
    return np.stack(E, 1), np.stack(Hs, 1)


def evaluate_error(ev, ew, E, Hh, dims: Dims, thetas, fA, fB, mat: MaterialOps):
    """``fun_no_inv/EvaluteError_Chiral_no_inv.m:10-36``: NFSEP residual
    ``norm(B x - w A x)`` and ORGSEP residual
    ``norm(B_mat*[C'*h; -C*e] - 1i*w*[e;h])`` with the explicit sparse curl."""
    C = curl_C(dims.shape, thetas, dims.mesh_len)
    CH = C.conj().T
    res_n, res_o = [], []
    for j in range(len(ew)):
        x = ev[:, j]
        res_n.append(np.linalg.norm(fB(x) - ew[j] * fA(x)))
        e, h = E[:, j], Hh[:, j]
        y1 = CH @ h
        y2 = -(C @ e)
        bm = np.concatenate([mat.N_int @ y1 + mat.J_int @ y2, mat.J_intH @ y1 + mat.M_int @ y2])
        res_o.append(np.linalg.norm(bm - 1j * ew[j] * np.concatenate([e, h])))
    return np.array(res_n), np.array(res_o)


# --------------------------------------------------------------------------
# Problem assembly for the benchmark configurations
# --------------------------------------------------------------------------
def woodpile_phases(gamma: float, eps_in=13.0):
    """Two phases: vacuum (phase 0) and a bi-isotropic rod (phase 1) with
    ``eps = eps_in*I``, ``mu = I``, ``xi = +1i*gamma*I``, ``zeta = -1i*gamma*I``."""
    I3 = np.eye(3)
    vac = Phase(I3.astype(np.complex128), I3.astype(np.complex128), np.zeros((3, 3), np.complex128),
                np.zeros((3, 3), np.complex128))
    rod = Phase(eps_in * I3 + 0j, I3 + 0j, 1j * gamma * I3, -1j * gamma * I3)
    return [vac, rod]


@dataclass
class BandProblem:
    dims: Dims
    thetas: tuple
    svd: SVDData
    fnc: Handles
    mat: MaterialOps
    inside: np.ndarray
    blocks: list = field(default_factory=list)  # per phase (N_cov, M_cov, J_cov)

    def A(self, x):
        return fncA(x, self.svd.Sigma_r)

    def B(self, x):
        return fncB(x, self.fnc, self.mat)


def build_problem(n, wave_vec=None, thetas=None, gamma=0.2, eps_in=13.0, width=0.25,
                  geometry="woodpile", phases=None, inside=None, A=None) -> BandProblem:
    """Set up one k-point as ``band_structure_woodpile_Lanczos_n60_gamma0p2.m:29-63``
    does: vertex rasterisation, two-phase material, SVD data, interpolated
    material operators and handles."""
    A = fcc_lattice() if A is None else A
    dims = Dims(n, n, n) if np.isscalar(n) else Dims(*n)
    if thetas is None:
        thetas = thetas_from_k(wave_vec, A)
    if inside is None:
        P = grid_vertices(dims) @ A.T          # Material_Locate_Isofunction.m:4-5
        if geometry == "woodpile":
            inside = woodpile_isofun(P, width, 1.0)
        elif geometry == "sphere":
            inside = sphere_isofun(P, np.zeros((1, 3)), width)
        else:
            raise ValueError(geometry)
    if phases is None:
        phases = woodpile_phases(gamma, eps_in)
    blocks = [material_blocks(ph, A) for ph in phases]
    Nv = dist_material(inside, blocks[0][0], blocks[1][0])
    Mv = dist_material(inside, blocks[0][1], blocks[1][1])
    Jv = dist_material(inside, blocks[0][2], blocks[1][2])
    svd = svd_matrix_generate(dims, thetas)
    Nint, Mint, Jint = interp_material_vertex(dims, thetas, Nv, Mv, Jv)
    return BandProblem(dims, tuple(thetas), svd, make_handles(svd), MaterialOps(Nint, Mint, Jint),
                       inside, blocks)


# --------------------------------------------------------------------------
# Per-vertex chiral fields and the eigenfrequency gradient (no reference
# counterpart: the reference places two-phase materials only; these restate
# the same assembly for per-vertex values and differentiate it)
# --------------------------------------------------------------------------
def field_diagonals(eps, gam, A=None):
    """Per-vertex covariant diagonals of ``eps I, mu = I, xi = i gamma I,
    zeta = -i gamma I``: ``material_blocks`` of each vertex in closed form,
    ``N = a G``, ``M = eps a G``, ``J = -i gamma a G`` with ``a = 1/(eps - gamma^2)``
    and ``G = A' A``.  Returns the 3x3 nested lists ``(Nv, Mv, Jv)`` that
    ``interp_material_vertex`` takes, and ``(a, b, g, G)``."""
    A = fcc_lattice() if A is None else A
    eps = np.asarray(eps, dtype=np.float64)
    gam = np.asarray(gam, dtype=np.float64)
    a = 1.0 / (eps - gam * gam)
    b = eps * a
    g = gam * a
    G = A.T @ A
    Nv = [[a * G[i, j] + 0j for j in range(3)] for i in range(3)]
    Mv = [[b * G[i, j] + 0j for j in range(3)] for i in range(3)]
    Jv = [[-1j * g * G[i, j] for j in range(3)] for i in range(3)]
    return (Nv, Mv, Jv), (a, b, g, G)


def build_problem_field(n, eps, gam, wave_vec=None, thetas=None, A=None) -> BandProblem:
    """``build_problem`` with per-vertex fields in place of the two phases."""
    A = fcc_lattice() if A is None else A
    dims = Dims(n, n, n)
    if thetas is None:
        thetas = thetas_from_k(wave_vec, A)
    (Nv, Mv, Jv), _ = field_diagonals(eps, gam, A)
    svd = svd_matrix_generate(dims, thetas)
    Nint, Mint, Jint = interp_material_vertex(dims, thetas, Nv, Mv, Jv)
    return BandProblem(dims, tuple(thetas), svd, make_handles(svd), MaterialOps(Nint, Mint, Jint),
                       np.zeros(dims.Nq, dtype=bool), [])


def material_quad_coeffs(dims: Dims, thetas, u, v):
    """Adjoint of ``interp_material_vertex``: per-vertex coefficient arrays
    ``cN[i][j]``, ``cM[i][j]``, ``cJ[i][j]`` such that, for per-vertex
    diagonals ``Nv``, ``Mv``, ``Jv``,

        u' M_int u = sum Re(Mv_ij * cM_ij),   v' N_int v = sum Re(Nv_ij * cN_ij),
        v' J_int u = sum Jv_ij * cJ_ij.

    Each assembled term ``L diag(A) R`` contributes ``conj(L' y_i) .* (R y_j)``;
    the factors are those of ``interp_material_vertex`` literally."""
    N = dims.Nq
    I = _I(N)
    C = [shift_diff(dims, thetas, d) for d in range(3)]
    CH = [c.conj().T.tocsr() for c in C]
    U = [u[i * N:(i + 1) * N] for i in range(3)]
    V = [v[i * N:(i + 1) * N] for i in range(3)]

    def k_of(i):
        return [d for d in range(3) if d != i]

    def term(Lfac, Rfac, yi, yj):
        return np.conj(Lfac.conj().T @ yi) * (Rfac @ yj)

    cN = [[None] * 3 for _ in range(3)]
    cM = [[None] * 3 for _ in range(3)]
    cJ = [[None] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(3):
            if i != j:
                cN[i][j] = term(0.25 * (2 * I + C[i]), 2 * I + CH[j], V[i], V[j])
            else:
                cN[i][i] = 0.5 * (np.conj(V[i]) * V[i] + term(I + C[i], I + CH[i], V[i], V[i]))
    for i in range(3):
        k = k_of(i)
        t1, t2 = (I + C[k[0]]), (I + C[k[1]])
        for j in range(3):
            if i == j:
                cM[i][i] = 0.25 * (np.conj(U[i]) * U[i] + term(t1, t1.conj().T, U[i], U[i])
                                   + term(t2, t2.conj().T, U[i], U[i])
                                   + term(t1 @ t2, t2.conj().T @ t1.conj().T, U[i], U[i]))
            else:
                l = k_of(j)
                cM[i][j] = term((1.0 / 16) * (2 * I + C[k[0]]) @ (2 * I + C[k[1]]),
                                (2 * I + CH[l[1]]) @ (2 * I + CH[l[0]]), U[i], U[j])
    for i in range(3):
        for j in range(3):
            k = k_of(j)
            cJ[i][j] = term(0.125 * (2 * I + C[i]), (2 * I + CH[k[1]]) @ (2 * I + CH[k[0]]), V[i], U[j])
    return cN, cM, cJ


def field_gradient(prob: BandProblem, x, omega, eps, gam, A=None):
    """FP64 reference gradient of one eigenfrequency with respect to the
    per-vertex fields: ``d omega/dp = omega x' (dB/dp) x / (x' B x)`` with
    ``x' B x = u' M_int u + v' N_int v + 2 Re(v' J_int u)`` (``fncB.m:3-6``,
    ``u = Pr x1``, ``v = Qr x2``), differentiated through the literal
    assembly via ``material_quad_coeffs``.  Returns ``(g_eps, g_gamma, xBx)``."""
    A = fcc_lattice() if A is None else A
    N = prob.dims.Nq
    x = np.asarray(x, dtype=np.complex128)
    u = prob.fnc.Pr(x[:2 * N])
    v = prob.fnc.Qr(x[2 * N:])
    cN, cM, cJ = material_quad_coeffs(prob.dims, prob.thetas, u, v)
    (_, _, _), (a, b, g, G) = field_diagonals(eps, gam, A)
    eps = np.asarray(eps, dtype=np.float64)
    gam = np.asarray(gam, dtype=np.float64)
    SN = sum(G[i, j] * cN[i][j].real for i in range(3) for j in range(3))
    SM = sum(G[i, j] * cM[i][j].real for i in range(3) for j in range(3))
    SJ = sum(G[i, j] * cJ[i][j].imag for i in range(3) for j in range(3))
    xbx = float(np.sum(a * SN + b * SM + 2.0 * g * SJ))
    a2 = a * a
    dq_de = -a2 * SN - gam * gam * a2 * SM - 2.0 * gam * a2 * SJ
    dq_dg = 2.0 * gam * a2 * SN + 2.0 * eps * gam * a2 * SM + 2.0 * a * (1.0 + 2.0 * gam * gam * a) * SJ
    s = omega / xbx
    return s * dq_de, s * dq_dg, xbx


def chiral_noise_field(n, seed=0, sigma=2.0, slope=8.0, eps_lo=1.0, eps_span=12.0, gamma_max=0.2):
    """Seeded smooth random medium on the n^3 vertices: s = sigmoid(slope *
    blur(N(0,1), sigma voxels)) with a periodic Gaussian blur (normalised to
    zero mean and unit standard deviation before the sigmoid), eps = eps_lo + eps_span s,
    gamma = gamma_max s.  Returns (eps, gamma), x fastest."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n))  # [z, y, x]
    k = np.fft.fftfreq(n) * 2 * np.pi
    kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
    filt = np.exp(-0.5 * sigma * sigma * (kx ** 2 + ky ** 2 + kz ** 2))
    sm = np.real(np.fft.ifftn(np.fft.fftn(w) * filt))
    sm = (sm - sm.mean()) / sm.std()
    s = 1.0 / (1.0 + np.exp(-slope * sm))
    s = s.reshape(-1)
    return eps_lo + eps_span * s, gamma_max * s


# --------------------------------------------------------------------------
# Implicitly restarted Lanczos (subroutines/Lanczos_gep.m)
# --------------------------------------------------------------------------
def gsreorthog(Q, fB, x):
    """``subroutines/Lanczos_gep.m:103-142``: B-orthogonalise ``x`` against
    the columns of ``Q`` by classical Gram-Schmidt repeated while the squared
    B-norm drops below half (Kahan-Parlett), with the reference's fallback to
    a unit vector.  Returns ``(p, r, tho)`` with ``x = Q r + tho p``."""
    n = Q.shape[1]
    r = np.zeros(n, dtype=np.complex128)
    tho = np.vdot(x, fB(x)).real
    if tho == 0:
        return np.zeros_like(x), r, 0.0
    mu = tho
    x_bar = x.copy()
    nrm = [np.vdot(Q[:, i], fB(Q[:, i])).real for i in range(n)]
    k = int(np.argmin(nrm))          # first index of the minimal B-norm (:117-125)
    ei = np.zeros(x.shape[0], dtype=np.complex128)
    ei[k] = 1.0
    eps = np.finfo(float).eps
    while True:
        s = Q.conj().T @ fB(x_bar)
        r = r + s
        x_bar = x_bar - Q @ s
        tau = np.vdot(x_bar, fB(x_bar)).real
        if tau / tho >= 0.5:
            break
        if tau > 0.1 * mu * eps:
            tho = tau
        else:
            tho = 0.1 * tho * eps
            mu = tho
            x_bar = ei.copy()
    tho = math.sqrt(np.vdot(x_bar, fB(x_bar)).real)
    return x_bar / tho, r, tho


def _implicit_restart(Q, alpha, beta, k, m, fB=None):
    """``Lanczos_gep.m:45-82``: m-k exact shifts at the Ritz values of smallest
    magnitude, band-truncated symmetrised QR steps, new length-k decomposition.
    The new residual vector is scaled by its Euclidean norm as ``:77`` does
    (``rho = norm(P)``); with ``fB`` given, by its B-norm instead, which keeps
    the basis B-orthonormal."""
    T = np.diag(alpha[:m]) + np.diag(beta[:m - 1], -1) + np.diag(beta[:m - 1], 1)
    ritz = np.linalg.eigvalsh(T)
    unwanted = ritz[np.argsort(np.abs(ritz), kind="stable")[:m - k]]
    e = np.zeros(m)
    e[m - 1] = 1.0
    I = np.eye(m)
    U_total = I.copy()
    for mu in unwanted:
        U, R = np.linalg.qr(T - mu * I)
        U_total = U_total @ U
        T = R @ U + mu * I
        for j in range(m - 2):
            T[j, j + 2:] = 0.0
        T = (T + T.T) / 2
    b = U_total.T @ e
    Qm = Q[:, :m] @ U_total
    P = T[k, k - 1] * Qm[:, k] + beta[m - 1] * b[k - 1] * Q[:, m]
    rho = np.linalg.norm(P) if fB is None else math.sqrt(np.vdot(P, fB(P)).real)
    Qn = np.zeros_like(Q)
    Qn[:, :k] = Qm[:, :k]
    Qn[:, k] = P / rho
    alpha = alpha.copy()
    beta = beta.copy()
    beta[:k] = np.concatenate([np.diag(T, -1)[:k - 1], [rho]])
    alpha[:k] = np.diag(T)[:k]
    return Qn, alpha, beta


def lanczos_gep(fA, fB, fBinv, n, k, m, itmax, tol, v0, bnorm_restart=False):
    """``subroutines/Lanczos_gep.m:1-27`` line by line: start vector
    ``v0/(v0' B v0)``, Lanczos steps ``alpha_j = Re(q_j' A q_j)``,
    ``r = B^{-1} A q_j - alpha_j q_j - beta_{j-1} q_{j-1}`` B-orthogonalised
    by ``gsreorthog``, implicit restarts, stop when ``|beta_k| < tol |alpha_k|``.
    Returns ``(EV, EW, nit)`` with EW ascending (eig of the k x k tridiagonal).
    ``bnorm_restart`` replaces the Euclidean scaling of the restart vector
    (``:77``) by the B-norm (see ``_implicit_restart``)."""
    Q = np.zeros((n, m + 1), dtype=np.complex128)
    v0 = np.asarray(v0, dtype=np.complex128)
    Q[:, 0] = v0 / np.vdot(v0, fB(v0)).real
    alpha = np.zeros(m)
    beta = np.zeros(m)

    def steps(Q, alpha, beta, k0):
        for j in range(k0, m):
            temp = fA(Q[:, j])
            alpha[j] = np.vdot(Q[:, j], temp).real
            r = fBinv(temp) - alpha[j] * Q[:, j]
            if j > 0:
                r = r - beta[j - 1] * Q[:, j - 1]
            Q[:, j + 1], _, beta[j] = gsreorthog(Q[:, :j + 1], fB, r)
        return Q, alpha, beta

    Q, alpha, beta = steps(Q, alpha, beta, 0)
    nit = 0
    while nit < itmax:
        nit += 1
        Q, alpha, beta = steps(Q, alpha, beta, k)
        Q, alpha, beta = _implicit_restart(Q, alpha, beta, k, m, fB if bnorm_restart else None)
        if abs(beta[k - 1]) < tol * abs(alpha[k - 1]):
            T = np.diag(alpha[:k]) + np.diag(beta[:k - 1], -1) + np.diag(beta[:k - 1], 1)
            ew, V = np.linalg.eigh(T)
            return Q[:, :k] @ V, ew, nit
    return None, None, nit


# --------------------------------------------------------------------------
# JD-SIRA with locking (light_locked_Huang/): Driver4, Locking4, the 'CL'
# Ritz choice of Choose_Ritz_Pair_Unsymm4 and the SIRA correction
# --------------------------------------------------------------------------
def gram_schmidt_ref(Y):
    """``light_locked_Huang/Gram_Schmidt.m:1-25``: modified Gram-Schmidt
    dropping columns of norm <= 1e-6.  Returns the orthonormal columns."""
    Y = np.array(Y, dtype=np.complex128, copy=True)
    nq = 0
    for k in range(Y.shape[1]):
        t = np.linalg.norm(Y[:, k])
        if abs(t) > 1.0e-6:
            Y[:, nq] = Y[:, k] / t
            for j in range(k + 1, Y.shape[1]):
                Y[:, j] = Y[:, j] - np.vdot(Y[:, nq], Y[:, j]) * Y[:, nq]
            nq += 1
    return Y[:, :nq]


def _close_within(a, b, tol, kmax):
    """``|a - b| <= 10^k tol`` for some k in -1..kmax (the ladder of
    Choose_Ritz_Pair_Unsymm4.m:30-37,62-69,92-99)."""
    return any(abs(a - b) <= 10.0 ** k * tol for k in range(-1, kmax + 1))


def choose_ritz_pair_cl(iteno, ew, ew_order, target, VRR, tol, rppd, locked):
    """``light_locked_Huang/Choose_Ritz_Pair_Unsymm4.m:1-302`` for
    ``Choose_Type = 'CL'`` (the drivers' choice) with ``target_org == target``:
    Ritz values that repeat locked eigenvalues are removed with their
    multiplicities (:24-166), candidates are the real Ritz values above the
    target (:176-186), the closest ``ewno <= rppd`` are taken in order
    (:236-272) and the rest of the restart block is filled by distance
    (:274-301).  Returns ``(ewno, ritz_ew, ritz_ev)`` (columns normalised)."""
    sort_ritz = np.array(ew, dtype=np.complex128, copy=True)
    if ew_order > 1 and len(locked):
        sort_ew = np.array(locked, dtype=np.complex128, copy=True)
        nl = len(sort_ew)
        mult_cn = np.zeros(nl, dtype=int)
        for i in range(nl):                                              # :25-50
            if sort_ew[i].real > -1.0e13:
                c = 1
                for i1 in range(i + 1, nl):
                    if sort_ew[i1].real > -1.0e13 and _close_within(sort_ew[i1], sort_ew[i], tol, 1):
                        c += 1
                        sort_ew[i1] = -1.0e14
                mult_cn[i] = c
        idx_w = np.zeros(iteno, dtype=int)                               # 1-based owner, 0 = first
        mult_w = np.zeros(iteno, dtype=int)
        for i in range(iteno):                                           # :56-82
            if idx_w[i] == 0:
                c = 1
                for i1 in range(i + 1, iteno):
                    if idx_w[i1] == 0 and _close_within(sort_ritz[i1], sort_ritz[i], tol, 1):
                        c += 1
                        idx_w[i1] = i + 1
                mult_w[i] = c
        for i in range(nl):                                              # :84-166
            if sort_ew[i].real <= -1.0e13:
                continue
            ind = None
            for i1 in range(iteno):
                if idx_w[i1] == 0 and _close_within(sort_ritz[i1], sort_ew[i], tol, 5):
                    ind = i1
                    break
            if ind is None:
                continue
            owned = [jj for jj in range(iteno) if idx_w[jj] == ind + 1]
            if mult_cn[i] >= mult_w[ind]:
                sort_ritz[ind] = 1.0e14
                for jj in owned:
                    sort_ritz[jj] = 1.0e14
            else:
                grp = [ind] + owned
                ld = [np.linalg.norm(VRR[ew_order - 1:iteno, g]) for g in grp]
                for _ in range(mult_cn[i]):
                    kk = int(np.argmin(ld))
                    sort_ritz[grp[kk]] = 1.0e14
                    ld[kk] = 1.0e14
            idx_w[ind] = -1
    cand, dist = [], []
    for i in range(iteno):                                               # :176-186 ('CL')
        if abs(sort_ritz[i]) < 1.0e10:
            e = ew[i]
            if (abs(e.real) < 1e-4 and e.imag > 1e-3) or (e.real > np.real(target) and abs(e.imag) < 1e-8):
                cand.append(i)
                dist.append(abs(e.real - np.real(target)))
    if not cand:                                                         # :218-224
        cand = list(range(iteno))
        dist = [abs(sort_ritz[i] - target) for i in range(iteno)]
    dist = np.array(dist, dtype=float)
    ewno = min(len(cand), rppd)
    picked, ritz_ew, ritz_ev = [], [], []
    for _ in range(ewno):                                                # :236-272
        k = int(np.argmin(dist))
        picked.append(cand[k])
        ritz_ew.append(ew[cand[k]])
        v = VRR[:iteno, cand[k]]
        ritz_ev.append(v / np.linalg.norm(v))
        dist[k] = 1.0e14
    if ewno < rppd:                                                      # :274-301
        rest = [i for i in range(iteno) if i not in picked and abs(sort_ritz[i]) < 1.0e10]
        rest.sort(key=lambda i: abs(ew[i] - target))
        for i in rest[:rppd - ewno]:
            ritz_ew.append(ew[i])
            v = VRR[:iteno, i]
            ritz_ev.append(v / np.linalg.norm(v))
        ewno += min(rppd - ewno, len(rest))
    return ewno, np.array(ritz_ew), np.stack(ritz_ev, axis=1)


def sira_correction(A, rhs, tol, maxit, B=None, shift=0.0):
    """``SIRA_solve_residual_LS_GEP.m:54`` with ``LS_solver = 'minres'``:
    MINRES on ``GEP_shift_mtx_prod_vec`` (``Jacobi_Davidson/GEP_shift_mtx_prod_vec.m:28-29``),
    which applies ``A`` alone (its ``- sigma*B`` term is commented out;
    ``shift`` restores it).  ``minres1`` is not in the reference tree, so
    SciPy's MINRES (relative tolerance ``tol``) stands in for it.
    Returns ``(t, iters)``."""
    import scipy.sparse.linalg as spla
    n = rhs.shape[0]

    def mv(v):
        v = np.asarray(v).ravel()
        y = A(v)
        return y - shift * B(v) if shift != 0.0 else y

    op = spla.LinearOperator((n, n), matvec=mv, dtype=np.complex128)
    its = [0]

    def cb(_):
        its[0] += 1

    t, _ = spla.minres(op, rhs, rtol=tol, maxiter=maxit, callback=cb)
    return t, its[0]


def jdsira_driver4(A, B, mtxdim, no_restart, ew_number, tol, initial_vec, target, ls_tol=1e-2, ls_maxit=30000,
                   shift=0.0, max_outer=6000):
    """``GEP_AB_Herm_JDSIRA_Driver4.m:12-80`` with
    ``GEP_AB_Herm_JDSIRA_Locking4.m:91-505`` (target type 'CL', correction
    'SIRA' by MINRES without preconditioner, as
    ``main_EIG_np_sphere_n60_gamma3p46427.m:111-125`` calls it with
    ``A = fncB``, ``B = fncA``): the ``ew_number`` eigenpairs of
    ``A x = theta B x`` selected by the 'CL' rule around ``target``.

    Per outer step: projected pencil ``eig(V'AV, V'BV)`` (:96-121), Ritz
    choice, unit Ritz vector and residual ``r = A u - theta B u`` (:181-185),
    acceptance at ``rsdl <= tol`` or after five steps in ``(tol, 10 tol]``
    (:198-208), else ``t = minres(A, r)`` orthogonalised against V by
    classical Gram-Schmidt and appended (:262-312); restart keeps the locked
    vectors, the current Ritz vector and three more (:327-345); after
    convergence the pair is locked with every other Ritz pair already below
    ``tol`` (:346-505).  Returns ``(EW, EV, stats)`` with ``stats`` the
    outer steps and MINRES iterations."""
    import scipy.linalg as sla
    rppd = max(4, initial_vec.shape[1] if initial_vec.ndim == 2 else 1)
    iv = initial_vec.reshape(mtxdim, -1).astype(np.complex128)
    init = np.zeros((mtxdim, ew_number + rppd - 1), dtype=np.complex128)
    init[:, :iv.shape[1]] = iv
    proj = iv.shape[1]
    locked_ew, EV = [], []
    outer_total, inner_total = 0, 0
    ew_order = 1
    while ew_order <= ew_number:
        # --- Locking4
        V = np.zeros((mtxdim, no_restart + 2), dtype=np.complex128)
        V[:, :proj] = init[:, :proj]
        stop = False
        no_near = 0
        dim_eigsp = len(locked_ew)
        ep = 1
        while ep <= max_outer and not stop:
            AV = np.stack([A(V[:, i]) for i in range(proj)], axis=1)
            BV = np.stack([B(V[:, i]) for i in range(proj)], axis=1)
            iteno = proj
            while iteno <= no_restart and not stop:
                # lower triangles of V'AV, V'BV, mirrored (:96-110)
                M = V[:, :iteno].conj().T @ AV[:, :iteno]
                Lm = V[:, :iteno].conj().T @ BV[:, :iteno]
                M = np.tril(M) + np.tril(M, -1).conj().T
                Lm = np.tril(Lm) + np.tril(Lm, -1).conj().T
                ew, VRR = sla.eig(M, Lm)
                ewno, ritz_ew, ritz_ev = choose_ritz_pair_cl(iteno, ew, ew_order, target, VRR, tol, rppd,
                                                             locked_ew)
                u = V[:, :iteno] @ ritz_ev[:, 0]
                u = u / np.linalg.norm(u)
                rv = A(u) - ritz_ew[0] * B(u)
                rsdl = np.linalg.norm(rv)
                no_near = no_near + 1 if (tol < rsdl <= 10.0 * tol) else 0
                if rsdl <= tol or no_near >= 5:
                    stop = True
                elif iteno + 1 <= dim_eigsp + no_restart:
                    t, its = sira_correction(A, rv, ls_tol, ls_maxit, B, shift)
                    inner_total += its
                    for j in range(iteno):
                        t = t - np.vdot(V[:, j], t) * V[:, j]
                    V[:, iteno] = t / np.linalg.norm(t)
                    AV = np.concatenate([AV, A(V[:, iteno])[:, None]], axis=1)
                    BV = np.concatenate([BV, B(V[:, iteno])[:, None]], axis=1)
                iteno += 1
                ep += 1
                outer_total += 1
            if not stop:                                                 # :327-345 restart
                iteno -= 1
                jj = min(rppd - 1, ew_number + rppd - 1)
                keep = V[:, :iteno] @ ritz_ev[:iteno, 1:jj + 1]
                W = np.concatenate([V[:, :dim_eigsp], u[:, None], keep], axis=1)
                Q = gram_schmidt_ref(W)
                proj = Q.shape[1]
                V[:, :] = 0
                V[:, :proj] = Q
                init[:, :proj] = Q
        # --- lock the converged pair and every other Ritz pair below tol (:346-505)
        others, conv = [], []
        for i in range(1, ewno):
            w = V[:, :iteno - 1] @ ritz_ev[:iteno - 1, i]
            w = w / np.linalg.norm(w)
            r_i = np.linalg.norm(A(w) - ritz_ew[i] * B(w))
            others.append(w)
            conv.append(r_i <= tol)
        Vl = [V[:, i] for i in range(dim_eigsp)]
        Vl.append(u / np.linalg.norm(u))
        EV.append(u / np.linalg.norm(u))
        locked_ew.append(ritz_ew[0])
        j = 0
        for w, c, ri in zip(others, conv, ritz_ew[1:]):
            if c:
                Vl.append(w)
                EV.append(w)
                locked_ew.append(ri)
                j += 1
        for w, c in zip(others, conv):
            if not c:
                Vl.append(w)
        Q = gram_schmidt_ref(np.stack(Vl, axis=1))
        proj = min(Q.shape[1], ew_number + rppd - 1)
        init[:, :proj] = Q[:, :proj]
        ew_order += j + 1
    EW = np.array(locked_ew[:ew_number])
    return EW, np.stack(EV[:ew_number], axis=1), {"outer": outer_total, "minres": inner_total}
