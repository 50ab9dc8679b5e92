"""Eigenfrequency gradients with respect to per-vertex chiral fields.

``Frequencies`` plays the role of a ``torch.autograd.Function`` around the
band solve of a field-mode plan: forward solves every k-point instance with
``fame_lanczos`` and keeps the eigenvectors; backward calls the library's
backward entry ``fame_eig_gradient`` (Hellmann-Feynman form, FP64).  Members
of a degenerate cluster (relative spread below ``cluster_tol``) share the mean
of their incoming weights, so only the cluster trace is differentiated.
"""
from __future__ import annotations

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def cluster_weights(omega, weight, cluster_tol=1e-8):
    """Average `weight` over clusters of `omega` closer than cluster_tol (relative)."""
    om = np.asarray(omega, dtype=np.float64)
    w = np.asarray(weight, dtype=np.float64).copy()
    order = np.argsort(om)
    i = 0
    while i < len(order):
        j = i + 1
        while j < len(order) and abs(om[order[j]] - om[order[j - 1]]) <= cluster_tol * abs(om[order[j]]):
            j += 1
        idx = order[i:j]
        w[idx] = w[idx].mean()
        i = j
    return w


def solve_bands(plan, nbands, tol=1e-10, prec="c128", inner_tol=1e-12, p=None):
    """Batched band solve of every instance (fame_band_solve with Ritz vectors);
    returns (omega [nk, nbands] ascending, [ev (nbands, 4Nq) per instance]).
    The restart size p defaults to max(2 nbands, 20): at Gamma the two shifted
    zero modes (lambda = 1/omega ~ 1e4 and beyond) stretch the spectrum of
    B^{-1}A, and a small Krylov space then separates the next bands slowly."""
    p = max(2 * nbands, 20) if p is None else p
    r = plan.band_solve(nbands, tol=tol, prec=prec, inner_tol=inner_tol, want_vectors=True, p=p)
    if r["status"] != 0:
        raise RuntimeError(f"band solve did not converge (status {r['status']})")
    oms, evs = [], []
    for k in range(plan.nk):
        order = np.argsort(r["omega"][k])
        oms.append(r["omega"][k][order])
        evs.append(r["ev"][k][torch.as_tensor(order, device=r["ev"].device)])
    return np.stack(oms), evs


def gradient(plan, evs, omega, weights, cluster_tol=1e-8):
    """sum_{k,b} weights[k,b] d omega[k,b] / d(eps, gamma): FP64 CUDA tensors (Nq,)."""
    g_e = torch.zeros(plan.Nq, dtype=torch.float64, device="cuda")
    g_g = torch.zeros_like(g_e)
    for k, ev in enumerate(evs):
        w = cluster_weights(omega[k], weights[k], cluster_tol)
        if not np.any(w):
            continue
        plan.eig_gradient(ev, omega[k], w, inst=k, out=(g_e, g_g), accumulate=True)
    return g_e, g_g


if torch is not None:
    class Frequencies(torch.autograd.Function):
        """omega[k, b] = Frequencies.apply(eps, gamma, plan, nbands, tol, prec):
        the `nbands` lowest eigenfrequencies of every instance of a field-mode
        plan, differentiable with respect to the per-vertex eps and gamma."""

        @staticmethod
        def forward(ctx, eps, gamma, plan, nbands, tol=1e-10, prec="c128"):
            plan.set_fields(eps, gamma)
            om, evs = solve_bands(plan, nbands, tol=tol, prec=prec)
            ctx.plan, ctx.evs, ctx.om = plan, evs, om
            ctx.dev = eps.device
            return torch.as_tensor(om, dtype=torch.float64, device=eps.device)

        @staticmethod
        def backward(ctx, grad_out):
            w = grad_out.detach().cpu().numpy()
            g_e, g_g = gradient(ctx.plan, ctx.evs, ctx.om, w)
            return g_e.to(ctx.dev), g_g.to(ctx.dev), None, None, None, None
