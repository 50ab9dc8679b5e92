"""MATLAB-shaped entry points mirroring the reference's handles, so code
written against ``fncA`` / ``fncB`` / ``fncinvB`` / ``MtxVecMul_FFT`` /
``Lanczos`` reads the same.  Each is a thin call into the CUDA library.
"""
from __future__ import annotations

import math

import numpy as np

from .plan import Plan
from .setup import bi_isotropic, bloch_angles, fcc_lattice, rasterize


def fncA(x, plan: Plan, inst=None):
    """fun_Lanczos/fncA.m:1-5."""
    return plan.apply_A(x, inst)


def fncB(x, plan: Plan, inst=None):
    """fun_Lanczos/fncB.m:1-7."""
    return plan.apply_B(x, inst)


def fncinvB(x, plan: Plan, tol=1e-12, maxit=10000, inst=None):
    """fun_Lanczos/fncinvB.m:1-5: the pcg flag is ignored, as there."""
    y, _, _ = plan.apply_Binv(x, tol, maxit, inst)
    return y


def MtxVecMul_FFT(vec_in, plan: Plan, istrans="notranspose", inst=None):
    """subroutines/MtxVecMul_FFT.m:1 for quasi-periodic grids (D = 1, P = R = I)."""
    if istrans not in ("notranspose", "transpose"):
        raise ValueError("istrans must be 'notranspose' or 'transpose'")
    return plan.transform(vec_in, 0 if istrans == "notranspose" else 1, inst)


def Lanczos(plan: Plan, k, tol=1e-10, maxiter=10000, p=None, v0=None, inst=0, prec="c128", inner_tol=1e-12):
    """fun_Lanczos/Lanczos.m:1: returns (ev, ew, iter) with ew the k largest
    eigenvalues of B^{-1}A (omega = 1./ew, band_structure...:83)."""
    r = plan.lanczos(k, tol, maxiter, p, v0, inst, prec, inner_tol)
    return r["ev"], r["ew"], int(r["stats"][0])


def Lanczos_gep(plan: Plan, eigen_wanted, option, inst=0, inner_tol=1e-12):
    """subroutines/Lanczos_gep.m: implicitly restarted Lanczos for
    fncA x = lambda fncB x in the B inner product, on the GPU handles of `plan`
    (instance `inst`; fncinvB = CG on fncB to `inner_tol`, as fncinvB.m).

    option: dict with m (subspace size), itmax, tol, v0 (host or CUDA vector)
    and optionally bnorm (default False).  As in the reference, the start vector
    is v0/(v0' B v0), Ritz values of smallest magnitude are the exact shifts,
    vectors are B-orthogonalised by gsreorthog, and the iteration stops when
    |beta_k| < tol |alpha_k|.  The reference scales the restart vector by its
    Euclidean norm (Lanczos_gep.m:77) although the basis is B-orthonormal,
    which limits the accuracy of the returned pairs; bnorm=True uses the B-norm.
    Returns (EV (k, L) complex128 CUDA tensor, EW ascending NumPy array, nit)."""
    import torch
    k = int(eigen_wanted)
    m = int(option["m"])
    itmax = int(option["itmax"])
    tol = float(option["tol"])
    bnorm = bool(option.get("bnorm", False))
    L_ = 4 * plan.Nq
    dev = "cuda"
    fA = lambda x: plan.apply_A(x, inst=inst)  # noqa: E731
    fB = lambda x: plan.apply_B(x, inst=inst)  # noqa: E731

    def fBinv(x):
        y, _, _ = plan.apply_Binv(x, tol=inner_tol, maxit=10000, inst=inst)
        return y

    def bdot(x, y):
        return torch.vdot(x, y).real.item()

    v0 = torch.as_tensor(option["v0"], dtype=torch.complex128, device=dev).reshape(-1)
    Q = torch.zeros((m + 1, L_), dtype=torch.complex128, device=dev)
    Q[0] = v0 / bdot(v0, fB(v0))
    alpha = np.zeros(m)
    beta = np.zeros(m)
    eps = np.finfo(float).eps

    def gsreorthog(Qj, x):
        # Lanczos_gep.m:103-142 (rows of Qj are the columns of the reference's Q)
        tho = bdot(x, fB(x))
        if tho == 0:
            return torch.zeros_like(x), 0.0
        mu = tho
        xb = x.clone()
        nrm = [bdot(Qj[i], fB(Qj[i])) for i in range(Qj.shape[0])]
        ei = torch.zeros_like(x)
        ei[int(np.argmin(nrm))] = 1.0
        while True:
            s = Qj.conj() @ fB(xb)
            xb = xb - s @ Qj
            tau = bdot(xb, fB(xb))
            if tau / tho >= 0.5:
                break
            if tau > 0.1 * mu * eps:
                tho = tau
            else:
                tho = 0.1 * tho * eps
                mu = tho
                xb = ei.clone()
        t = math.sqrt(bdot(xb, fB(xb)))
        return xb / t, t

    def steps(k0):
        for j in range(k0, m):
            temp = fA(Q[j])
            alpha[j] = bdot(Q[j], temp)
            r = fBinv(temp) - alpha[j] * Q[j]
            if j > 0:
                r = r - beta[j - 1] * Q[j - 1]
            Q[j + 1], beta[j] = gsreorthog(Q[:j + 1], r)

    def restart():
        # Lanczos_gep.m:45-82
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
        Ut = torch.as_tensor(U_total, dtype=torch.complex128, device=dev)
        Qm = Ut.T @ Q[:m]
        P = T[k, k - 1] * Qm[k] + beta[m - 1] * b[k - 1] * Q[m]
        rho = math.sqrt(bdot(P, fB(P))) if bnorm else torch.linalg.vector_norm(P).item()
        Q[:k] = Qm[:k]
        Q[k] = P / rho
        Q[k + 1:] = 0
        beta[:k] = np.concatenate([np.diag(T, -1)[:k - 1], [rho]])
        alpha[:k] = np.diag(T)[:k]

    steps(0)
    nit = 0
    while nit < itmax:
        nit += 1
        steps(k)
        restart()
        if abs(beta[k - 1]) < tol * abs(alpha[k - 1]):
            T = np.diag(alpha[:k]) + np.diag(beta[:k - 1], -1) + np.diag(beta[:k - 1], 1)
            ew, V = np.linalg.eigh(T)
            Vt = torch.as_tensor(V, dtype=torch.complex128, device=dev)
            return Vt.T @ Q[:k], ew, nit
    return None, None, nit


def woodpile_plan(n: int, wave_vecs, gamma=0.2, eps_in=13.0, width=0.25, gammas=None) -> Plan:
    """Plan for the woodpile benchmark: FCC a=1, rods of width `width`
    (Public/woodpile_isofun.m convention), inside eps*I, mu=I, xi=+i*gamma*I,
    zeta=-i*gamma*I, vacuum outside; one instance per wave vector.  `gammas`
    gives one chirality per instance."""
    A = fcc_lattice()
    kv = np.atleast_2d(np.asarray(wave_vecs, dtype=np.float64))
    th = np.stack([bloch_angles(k, A) for k in kv])
    phase = rasterize(n, "woodpile", width, A)
    vac = bi_isotropic(1.0, 0.0)
    if gammas is None:
        return Plan.from_phases(n, th, phase, [vac, bi_isotropic(eps_in, gamma)], A)
    gs = np.broadcast_to(np.asarray(gammas, dtype=np.float64), (kv.shape[0],))
    return Plan.from_phases(n, th, phase, [[vac, bi_isotropic(eps_in, g)] for g in gs], A)
