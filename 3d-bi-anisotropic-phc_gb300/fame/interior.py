"""Interior eigenpairs of inclusion crystals by shifted SIRA.

The reference's light-localisation scripts (main_EIG_np_sphere_n60_gamma3p46427.m,
main_EIG_np_tri_n60_gamma*.m) place one chiral inclusion in the FCC cell,
call GEP_AB_Herm_JDSIRA_Driver4(fncB, fncA, ...) for the eigenfrequencies
closest to a target, restore the fields and report the field maxima outside
the inclusion (draw_test/Fig6cd_plot_max_field.m).  Here the inclusion is a
sphere or a regular tetrahedron at the cell origin, the target is a multiple
of the 4th band edge at Gamma, the correction equation is the shifted one
(B - sigma A) t = r solved in complex64 by MINRES, and the outer iteration,
locking and residual checks run in FP64 (fame_jdsira); the fields, ORGSEP
residuals and maxima come from fame_restore.

Command line: ``python -m fame.interior_cli --shape sphere --gamma 3.46427 --n 60``.
"""
from __future__ import annotations

import time

import numpy as np

from .plan import Plan
from .setup import bi_isotropic, bloch_angles, fcc_lattice, rasterize

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def inclusion_plan(n, wave_vecs, shape="sphere", gamma=0.5, eps_in=13.0, size=None):
    """Plan with vacuum outside and eps*I, mu = I, xi = -zeta = i*gamma*I inside a
    sphere (radius `size`, default 0.25a) or regular tetrahedron (edge `size`,
    default 0.5a) at the cell origin; one instance per wave vector."""
    A = fcc_lattice()
    if shape == "sphere":
        phase = rasterize(n, "sphere", 0.25 if size is None else size, A)
    elif shape in ("tetra", "tri", "tetrahedron"):
        phase = rasterize(n, "tetra", 0.5 if size is None else size, A)
    else:
        raise ValueError(shape)
    kv = np.atleast_2d(np.asarray(wave_vecs, dtype=np.float64))
    th = np.stack([bloch_angles(k, A) for k in kv])
    return Plan.from_phases(n, th, phase, [bi_isotropic(1.0, 0.0), bi_isotropic(eps_in, gamma)], A)


def band_edge(plan, band=4, tol=1e-10, prec="c64"):
    """omega of the `band`-th lowest band of instance 0."""
    r = plan.lanczos(band, tol=tol, prec=prec, inst=0, p=max(2 * band, 20), want_vectors=False)
    return float(np.sort(r["omega"])[band - 1])


def interior_modes(plan, nev, sigma, tol=1e-8, inner_tol=1e-3, no_restart=50, restart_dim=4, inner_prec="c64",
                   outside_only=True):
    """The `nev` eigenfrequencies of instance 0 closest to `sigma` (shifted SIRA,
    shift = sigma) with NFSEP and ORGSEP residuals and field maxima."""
    t0 = time.perf_counter()
    plan.set_option("sira_nearest", 1)  # the pairs nearest sigma, on either side
    r = plan.jdsira(nev, target=sigma, shift=sigma, tol=tol, no_restart=no_restart, restart_dim=restart_dim,
                    inner_tol=inner_tol, inner_prec=inner_prec, want_vectors=True)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ok = np.isfinite(r["ew"])
    out = dict(omega=r["ew"], res_nfsep=r["res"], stats=r["stats"], status=r["status"], t_sira=t1 - t0)
    if np.any(ok):
        idx = torch.as_tensor(np.where(ok)[0], device=r["ev"].device)
        rs = plan.restore(r["ev"][idx], r["ew"][ok], want_fields=False, outside_only=outside_only)
        torch.cuda.synchronize()
        out.update(res_orgsep=rs["res_orgsep"], max_e=rs["max_e"], max_h=rs["max_h"],
                   t_restore=time.perf_counter() - t1)
    return out
