"""fame_apply_B_noalloc: fncB for callers that cannot let the library allocate
device memory at call time (a MEX gateway under MATLAB's gpuArray memory
manager, an application pooling its whole device budget).  It draws its
scratch from one fixed 16 MiB device array instead of the plan's on-demand
scratch.  Checked through the C ABI against fame_apply_B on two calls in a
row (the array keeps the previous call's contents between them)."""
import ctypes as C

import pytest

import fame
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


def test_noalloc_rejects_oversized(cuda, fame_lib):
    import torch

    plan = fame.woodpile_plan(60, [fame.fcc_point("X")])
    x = torch.zeros((1, 4 * 60 ** 3), dtype=torch.complex64, device="cuda")
    with pytest.raises(fame.FameError) as e:
        _noalloc(plan, x)
    assert e.value.code == 1 and "16777216" in str(e.value)
    plan.close()
