"""Field-mode plans (per-vertex eps, gamma) and the backward entry
fame_eig_gradient on the GPU, against the oracle: fncB parity with the literal
sparse assembly, the gradient against the oracle's FP64 reference gradient on
the same eigenvectors, the autograd wrapper against a directional finite
difference of GPU band solves, and the adjoint workload at n = 40 (8 k-points
on Gamma-X-W-L, gap between bands 2 and 3, 32 seeded voxels)."""
import numpy as np
import pytest
import torch

import fame
import oracle as O

pytestmark = pytest.mark.gpu


def field_setup(n, labels, seed=0, sigma=1.0):
    A = fame.fcc_lattice()
    kv = [fame.fcc_point(lab) for lab in labels]
    th = np.stack([fame.bloch_angles(k, A) for k in kv])
    eps, gam = O.chiral_noise_field(n, seed=seed, sigma=sigma)
    return th, eps, gam


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-12), (torch.complex64, 2e-5)])
def test_field_fncB_matches_oracle(cuda, fame_lib, dtype, tol):
    n = 8
    th, eps, gam = field_setup(n, ("X", "W"))
    plan = fame.Plan.from_fields(n, th, eps, gam)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, 4 * n ** 3)) + 1j * rng.standard_normal((2, 4 * n ** 3))
    y = plan.apply_B(torch.as_tensor(x).to(dtype).cuda()).cpu().numpy()
    for k in range(2):
        P = O.build_problem_field(n, eps, gam, thetas=th[k])
        ref = P.B(x[k])
        assert np.linalg.norm(y[k] - ref) <= tol * np.linalg.norm(ref)


def test_set_fields_rejects_non_definite(cuda, fame_lib):
    n = 4
    th, eps, gam = field_setup(n, ("X",))
    plan = fame.Plan.from_fields(n, th, eps, gam)
    bad = gam.copy()
    bad[5] = 10.0  # eps - gamma^2 < 0
    with pytest.raises(fame.FameError):
        plan.set_fields(eps, bad)


def test_gradient_matches_oracle_reference(cuda, fame_lib):
    n = 8
    th, eps, gam = field_setup(n, ("X", "W"), seed=2)
    plan = fame.Plan.from_fields(n, th, eps, gam)
    om, evs = fame.adjoint.solve_bands(plan, 4, tol=1e-11)
    for k in range(2):
        w = np.array([0.0, -1.0, 1.0, 0.0])  # gap between bands 2 and 3
        g_e, g_g, xbx = plan.eig_gradient(evs[k], om[k], w, inst=k)
        assert np.allclose(xbx, 1.0, atol=1e-9)  # B-normalised Ritz vectors
        P = O.build_problem_field(n, eps, gam, thetas=th[k])
        X = evs[k].cpu().numpy()
        re = np.zeros(n ** 3)
        rg = np.zeros(n ** 3)
        for b in (1, 2):
            e_, g_, xb = O.field_gradient(P, X[b], om[k][b], eps, gam)
            assert abs(xb - xbx[b]) <= 1e-10
            re += w[b] * e_
            rg += w[b] * g_
        ge, gg = g_e.cpu().numpy(), g_g.cpu().numpy()
        assert np.abs(ge - re).max() <= 1e-10 * np.abs(re).max()
        assert np.abs(gg - rg).max() <= 1e-10 * np.abs(rg).max()


def test_autograd_directional_difference(cuda, fame_lib):
    n = 8
    th, eps, gam = field_setup(n, ("X", "L"), seed=4)
    plan = fame.Plan.from_fields(n, th, eps, gam)
    e = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    g = torch.tensor(gam, dtype=torch.float64, requires_grad=True)
    om = fame.adjoint.Frequencies.apply(e, g, plan, 4, 1e-12, "c128")
    J = (om[:, 2] - om[:, 1]).sum()
    J.backward()
    rng = np.random.default_rng(9)
    de = rng.standard_normal(n ** 3)
    dg = 0.1 * rng.standard_normal(n ** 3)
    lin = float(e.grad.numpy() @ de + g.grad.numpy() @ dg)
    h = 1e-4

    def gap(s):
        o = fame.adjoint.Frequencies.apply(torch.tensor(eps + s * de), torch.tensor(gam + s * dg), plan, 4, 1e-12,
                                           "c128")
        return float((o[:, 2] - o[:, 1]).sum())

    fd = (gap(h) - gap(-h)) / (2 * h)
    assert abs(fd - lin) <= 1e-5 * abs(lin), (fd, lin)


def test_adjoint_workload_n40(cuda, fame_lib):
    """n = 40: eps = 1 + 12 s, gamma = 0.2 s with s a seeded smooth sigmoid
    field; objective sum over 8 k-points on Gamma-X-W-L of omega_3 - omega_2;
    mixed-precision band solves, FP64 gradient; 32 seeded voxels against the
    oracle's FP64 reference gradient on the same eigenvectors (two k-points)."""
    n = 40
    A = fame.fcc_lattice()
    kv = fame.band_path(labels=("G", "X", "W", "L"), npts=8)
    th = np.stack([fame.bloch_angles(k, A) for k in kv])
    eps, gam = O.chiral_noise_field(n, seed=0)
    plan = fame.Plan.from_fields(n, th, eps, gam)
    om, evs = fame.adjoint.solve_bands(plan, 4, tol=1e-10, prec="c64")
    w = np.zeros((8, 4))
    w[:, 1], w[:, 2] = -1.0, 1.0
    g_e, g_g = fame.adjoint.gradient(plan, evs, om, w)
    assert torch.isfinite(g_e).all() and torch.isfinite(g_g).all()
    vox = np.random.default_rng(11).choice(n ** 3, 32, replace=False)
    for k in (1, 5):
        ge_k, gg_k, _ = plan.eig_gradient(evs[k], om[k], w[k], inst=k)
        P = O.build_problem_field(n, eps, gam, thetas=th[k])
        X = evs[k].cpu().numpy()
        re = np.zeros(n ** 3)
        rg = np.zeros(n ** 3)
        for b in (1, 2):
            e_, g_, _ = O.field_gradient(P, X[b], om[k][b], eps, gam)
            re += w[k, b] * e_
            rg += w[k, b] * g_
        ge, gg = ge_k.cpu().numpy()[vox], gg_k.cpu().numpy()[vox]
        assert np.all(np.abs(ge - re[vox]) <= 1e-5 * np.abs(re[vox]) + 1e-12 * np.abs(re).max())
        assert np.all(np.abs(gg - rg[vox]) <= 1e-5 * np.abs(rg[vox]) + 1e-12 * np.abs(rg).max())
