"""fame_apply_B_noalloc: fncB for callers that cannot let the library allocate
device memory at call time (a MEX gateway under MATLAB's gpuArray memory
manager, an application pooling its whole device budget).  It draws its
scratch from one fixed 16 MiB device array instead of the plan's on-demand
scratch.  Checked through the C ABI against fame_apply_B on two calls in a
row (the array keeps the previous call's contents between them), against
the oracle's fncB (fun_Lanczos/fncB.m:3-6), and on a plan whose fncB runs in
sub-batches (the layout that places the second work buffer inside the fixed
array)."""
import ctypes as C

import numpy as np
import pytest

import fame
import oracle as O
from problems import Pair, relerr

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 2e-5}


def _noalloc(plan, x):
    import torch

    lib = fame.load()
    y = torch.empty_like(x)
    lib.fame_set_stream(plan.raw, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    prec = 0 if x.dtype == torch.complex128 else 1
    rc = lib.fame_apply_B_noalloc(plan.raw, prec, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                  x.shape[0])
    fame._lib.check(rc, plan.raw, "fame_apply_B_noalloc")
    return y


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_noalloc_matches_apply_B_twice(cuda, fame_lib, prec):
    import torch

    dt = torch.complex128 if prec == "c128" else torch.complex64
    P = Pair(12, nk=2, seed=21)
    for call in range(2):  # two calls in a row: the shared scratch holds the previous call's data
        x = torch.from_numpy(P.vec(4 * P.Nq, 3)).to(device="cuda", dtype=dt)
        ref = P.plan.apply_B(x).cpu().numpy()
        got = _noalloc(P.plan, x).cpu().numpy()
        torch.cuda.synchronize()
        assert relerr(got, ref) < TOL[prec], (call, relerr(got, ref))
        xh = x.cpu().numpy().astype(np.complex128)
        for v in range(xh.shape[0]):
            svd, fnc, mat = P.ref(v % P.nk)
            assert relerr(got[v], O.fncB(xh[v], fnc, mat)) < TOL[prec], (call, v)


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_noalloc_sub_batches(cuda, fame_lib, prec):
    """fncB in sub-batches of 2 vectors (as the autotuner may choose), so each
    sub-batch reuses the front of both work buffers of the fixed array."""
    import torch

    dt = torch.complex128 if prec == "c128" else torch.complex64
    P = Pair(12, nk=3, seed=5)
    P.plan.set_tune(prec, 6, 2, 0)
    for call in range(2):
        x = torch.from_numpy(P.vec(4 * P.Nq, 6)).to(device="cuda", dtype=dt)
        ref = P.plan.apply_B(x).cpu().numpy()
        got = _noalloc(P.plan, x).cpu().numpy()
        assert relerr(got, ref) < TOL[prec], (call, relerr(got, ref))
    P.plan.set_tune(prec, 6, 0, 256)
    x = torch.from_numpy(P.vec(4 * P.Nq, 6)).to(device="cuda", dtype=dt)
    t = P.plan.autotune(6, prec=prec)
    got = _noalloc(P.plan, x).cpu().numpy()
    assert relerr(got, P.plan.apply_B(x).cpu().numpy()) < TOL[prec], t


def test_noalloc_null_plan_sets_error(cuda, fame_lib):
    lib = fame.load()
    rc = lib.fame_apply_B_noalloc(None, 1, None, None, 1)
    assert rc == 1
    assert b"null plan" in lib.fame_last_error(None)


def test_noalloc_rejects_oversized(cuda, fame_lib):
    import torch

    plan = fame.woodpile_plan(60, [fame.fcc_point("X")])
    x = torch.zeros((1, 4 * 60 ** 3), dtype=torch.complex64, device="cuda")
    with pytest.raises(fame.FameError) as e:
        _noalloc(plan, x)
    assert e.value.code == 1 and "16777216" in str(e.value)
    plan.close()
