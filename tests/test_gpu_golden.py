"""The CUDA library against the committed golden fixtures of the woodpile
problem (the oracle's outputs, tests/golden/make_golden.py): fncB, fncA and
MtxVecMul_FFT in complex128 (1e-12) and complex64 (2e-5), FP64 Lanczos
eigenvalues (1e-10 relative) and the device rasteriser's vertex ids
(exactly)."""
import numpy as np
import pytest

import fame
from golden import make_golden as G

pytestmark = pytest.mark.gpu

FIX = np.load(G.FILE)
TOL = {"c128": 1e-12, "c64": 2e-5}


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(x, prec):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(
        device="cuda", dtype=torch.complex128 if prec == "c128" else torch.complex64)


@pytest.mark.parametrize("n,label", G.CASES)
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_operators_match_fixture(cuda, fame_lib, n, label, prec):
    key = f"n{n}_{label}"
    plan = fame.woodpile_plan(n, [fame.fcc_point(label)])
    Nq = n ** 3
    x = G.det_vec(4 * Nq, n)
    y3 = G.det_vec(3 * Nq, n + 1)
    assert relerr(plan.apply_B(dev(x, prec)).cpu().numpy(), FIX[key + "_Bx"]) < TOL[prec]
    assert relerr(plan.apply_A(dev(x, prec)).cpu().numpy(), FIX[key + "_Ax"]) < TOL[prec]
    tn = fame.MtxVecMul_FFT(dev(y3, prec), plan, "notranspose").cpu().numpy()
    tt = fame.MtxVecMul_FFT(dev(y3, prec), plan, "transpose").cpu().numpy()
    assert relerr(tn, FIX[key + "_Tn"]) < TOL[prec]
    assert relerr(tt, FIX[key + "_Tt"]) < TOL[prec]


@pytest.mark.parametrize("n,label", G.EIG_CASES)
def test_lanczos_matches_fixture(cuda, fame_lib, n, label):
    plan = fame.woodpile_plan(n, [fame.fcc_point(label)])
    r = plan.lanczos(G.BANDS, tol=1e-10, maxit=10000, p=2 * G.BANDS, prec="c128", want_vectors=False)
    assert r["status"] == 0
    assert np.allclose(r["ew"], FIX[f"n{n}_{label}_ew"], rtol=1e-10, atol=0)


def test_rasteriser_matches_fixture(cuda, fame_lib):
    n = G.RASTER_N
    for name, shape, size in (("woodpile", "woodpile", 0.25), ("sphere", "sphere", 0.25), ("tetra", "tetra", 0.5)):
        ref = np.unpackbits(FIX[f"raster_{name}"])[:n ** 3]
        got = fame.rasterize(n, shape, size)
        assert np.array_equal(got, ref), name
    for n_, lab in G.CASES:
        got = fame.rasterize(n_, "woodpile", 0.25)
        assert np.array_equal(got, FIX[f"n{n_}_{lab}_inside"])


def test_first_workload_n24_matches_fixture(cuda, fame_lib):
    """The woodpile at n = 24, X point, 10 bands (the reference's own
    CPU-sized case): the FP64 form equals the oracle's Lanczos.m
    (tests/golden/woodpile_n24_X.npz) to 1e-10, the mixed form to 1e-8."""
    ref = np.load(G.N24_FILE)["ew"]
    plan = fame.woodpile_plan(24, [fame.fcc_point("X")])
    r = plan.lanczos(10, tol=1e-10, maxit=10000, p=20, prec="c128", want_vectors=False)
    assert r["status"] == 0
    assert np.allclose(r["ew"], ref, rtol=1e-10, atol=0), (r["ew"], ref)
    m = plan.band_solve(10, tol=1e-10, prec="c64", inner_tol=1e-11, p=26)
    assert m["status"] == 0
    assert np.allclose(m["ew"][0], ref, rtol=1e-8, atol=0), (m["ew"][0], ref)
    assert m["res"].max() <= 1e-8
