"""fncB in double-single (float-float) arithmetic (FAME_C128_DS): complex128
vectors in and out, every operation inside as an unevaluated pair of floats
(~48 significant bits) on the FP32 pipes.  The mixed inner solves take their
residuals b - B x through it (FAME_OPT_DS_RESIDUAL).  Checked against the
complex128 fncB (fun_Lanczos/fncB.m:3-6) and the oracle, in phase-table and
field mode, and through a mixed band solve with and without it."""
import ctypes as C

import numpy as np
import pytest

import fame
import oracle as O
from problems import Pair, relerr

pytestmark = pytest.mark.gpu

DS = 2  # FAME_C128_DS


def _apply_ds(plan, x, inst=None):
    import torch

    lib = fame.load()
    y = torch.empty_like(x)
    lib.fame_set_stream(plan.raw, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    ip = None
    if inst is not None:
        ia = (C.c_int * len(inst))(*[int(i) for i in inst])
        ip = C.cast(ia, C.POINTER(C.c_int))
    rc = lib.fame_apply_B(plan.raw, DS, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), x.shape[0], ip, 0)
    fame._lib.check(rc, plan.raw, "fame_apply_B")
    torch.cuda.synchronize()
    return y


def test_ds_fncB_matches_complex128_and_oracle_n12(cuda, fame_lib):
    import torch

    P = Pair(12, nk=2, seed=33)
    x = torch.from_numpy(P.vec(4 * P.Nq, 3)).to(device="cuda", dtype=torch.complex128)
    ref = P.plan.apply_B(x).cpu().numpy()
    got = _apply_ds(P.plan, x).cpu().numpy()
    assert relerr(got, ref) < 1e-13, relerr(got, ref)
    xh = x.cpu().numpy()
    for v in range(xh.shape[0]):
        svd, fnc, mat = P.ref(v % P.nk)
        assert relerr(got[v], O.fncB(xh[v], fnc, mat)) < 1e-12


def test_ds_fncB_matches_complex128_n60(cuda, fame_lib):
    import torch

    n = 60
    plan = fame.woodpile_plan(n, fame.band_path(npts=40)[[0, 9, 39]])
    rng = np.random.default_rng(5)
    x = rng.standard_normal((3, 4 * n ** 3)) + 1j * rng.standard_normal((3, 4 * n ** 3))
    xt = torch.from_numpy(x).cuda()
    ref = plan.apply_B(xt).cpu().numpy()
    got = _apply_ds(plan, xt).cpu().numpy()
    assert relerr(got, ref) < 1e-13, relerr(got, ref)
    # instance indices are honoured: vector 0 as instance 2
    got2 = _apply_ds(plan, xt[:1].contiguous(), inst=[2]).cpu().numpy()
    ref2 = plan.apply_B(xt[:1].contiguous(), inst=2).cpu().numpy()
    assert relerr(got2, ref2) < 1e-13
    plan.close()


def test_ds_fncB_field_mode(cuda, fame_lib):
    """Per-vertex fields (fame_plan_create_field): the double-single tables
    follow the fields."""
    import torch

    n = 12
    rng = np.random.default_rng(9)
    eps = 1.0 + 12.0 * rng.random(n ** 3)
    gam = 0.3 * rng.random(n ** 3)
    th = np.stack([fame.bloch_angles(fame.fcc_point(lab), fame.fcc_lattice()) for lab in ("X", "L")])
    plan = fame.Plan.from_fields(n, th, eps, gam)
    x = rng.standard_normal((2, 4 * n ** 3)) + 1j * rng.standard_normal((2, 4 * n ** 3))
    xt = torch.from_numpy(x).cuda()
    ref = plan.apply_B(xt).cpu().numpy()
    got = _apply_ds(plan, xt).cpu().numpy()
    assert relerr(got, ref) < 1e-13, relerr(got, ref)
    plan.close()


def test_ds_unsupported_grid(cuda, fame_lib):
    import torch

    plan = fame.woodpile_plan(32, [fame.fcc_point("X")])
    x = torch.zeros(1, 4 * 32 ** 3, dtype=torch.complex128, device="cuda")
    lib = fame.load()
    y = torch.empty_like(x)
    rc = lib.fame_apply_B(plan.raw, DS, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), 1, None, 0)
    assert rc == fame._lib.FAME_ERR_UNSUPPORTED
    assert b"double-single" in lib.fame_last_error(plan.raw)
    plan.close()


def test_mixed_band_solve_with_ds_residuals(cuda, fame_lib):
    """The mixed form with the double-single residuals against FP64 ones:
    the same eigenvalues to rounding, residuals below the bar."""
    n, k = 12, 6
    plan = fame.woodpile_plan(n, [fame.fcc_point("X"), fame.fcc_point("L")])
    out = {}
    for ds in (0, 1):
        plan.set_option("ds_residual", ds)
        out[ds] = plan.band_solve(k, tol=1e-8, prec="c64", inner_tol=3e-12, p=2 * k + 4)
        assert out[ds]["status"] == 0
        assert out[ds]["res"].max() <= 1e-8
    assert np.allclose(out[1]["ew"], out[0]["ew"], rtol=1e-10, atol=0)
    plan.close()


def test_ds_lanes_and_autotune(cuda, fame_lib):
    """Every compiled FFT split of the double-single plane kernels and both
    stencil forms give the complex128 operator to 1e-13; the autotuner
    times them and reports a compiled choice."""
    import torch

    n = 60
    plan = fame.woodpile_plan(n, fame.band_path(npts=40)[[3, 17]])
    rng = np.random.default_rng(6)
    x = rng.standard_normal((2, 4 * n ** 3)) + 1j * rng.standard_normal((2, 4 * n ** 3))
    xt = torch.from_numpy(x).cuda()
    ref = plan.apply_B(xt).cpu().numpy()
    for tpb in (0, 256):
        for lanes in (-1, 3, 4, 5, 0):
            plan.set_tune("c128ds", 2, 0, tpb, lanes)
            got = _apply_ds(plan, xt).cpu().numpy()
            assert relerr(got, ref) < 1e-13, (tpb, lanes, relerr(got, ref))
    t = plan.autotune(nvec=2, prec="c128ds")
    assert t["lanes"] in (-1, 3, 4, 5) and t["us"] > 0
    plan.close()


@pytest.mark.parametrize("n", [24, 40, 48])
def test_ds_fncB_other_grids(cuda, fame_lib, n):
    """Every other grid with a compiled double-single fncB against the
    complex128 operator."""
    import torch

    plan = fame.woodpile_plan(n, [fame.fcc_point("X"), fame.fcc_point("W")])
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, 4 * n ** 3)) + 1j * rng.standard_normal((2, 4 * n ** 3))
    xt = torch.from_numpy(x).cuda()
    ref = plan.apply_B(xt).cpu().numpy()
    got = _apply_ds(plan, xt).cpu().numpy()
    assert relerr(got, ref) < 1e-13, relerr(got, ref)
    plan.close()
