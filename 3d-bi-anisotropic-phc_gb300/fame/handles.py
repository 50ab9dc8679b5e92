"""MATLAB-shaped entry points mirroring the reference's handles, so code
written against ``fncA`` / ``fncB`` / ``fncinvB`` / ``MtxVecMul_FFT`` /
``Lanczos`` reads the same.  Each is a thin call into the CUDA library.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from .plan import Plan
from .setup import bi_isotropic, bloch_angles, fcc_lattice, vertex_positions, woodpile_inside


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


def woodpile_plan(n: int, wave_vecs, gamma=0.2, eps_in=13.0, width=0.25, gammas=None) -> Plan:
    """Plan for the woodpile benchmark: FCC a=1, rods of width `width`
    (Public/woodpile_isofun.m convention), inside eps*I, mu=I, xi=+i*gamma*I,
    zeta=-i*gamma*I, vacuum outside; one instance per wave vector.  `gammas`
    gives one chirality per instance."""
    A = fcc_lattice()
    kv = np.atleast_2d(np.asarray(wave_vecs, dtype=np.float64))
    th = np.stack([bloch_angles(k, A) for k in kv])
    inside = woodpile_inside(vertex_positions(n, A), width)
    phase = inside.astype(np.uint8)
    vac = bi_isotropic(1.0, 0.0)
    if gammas is None:
        return Plan.from_phases(n, th, phase, [vac, bi_isotropic(eps_in, gamma)], A)
    gs = np.broadcast_to(np.asarray(gammas, dtype=np.float64), (kv.shape[0],))
    return Plan.from_phases(n, th, phase, [[vac, bi_isotropic(eps_in, g)] for g in gs], A)
