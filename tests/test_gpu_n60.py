"""The CUDA library against the oracle at the benchmark's own size: the
woodpile at n = 60 (vectors of 6·60³ complex entries), X and L points.

The fixtures (tests/golden/make_golden.py --n60ops / --n60eig) hold the
oracle's outputs on closed-form inputs.  A complex128 vector at n = 60 is
13.8 MB, so each output is stored as a digest (1024 sampled values, four
sketch inner products over every entry, the norm) and the library's output
is reduced the same way.

* operators (fncB, fncA, MtxVecMul_FFT both ways, Pr / Qr / Prs / Qrs):
  complex128 within 1e-12, complex64 within 2e-5 (fun_Lanczos/fncB.m:3-6,
  subroutines/MtxVecMul_FFT.m:18-62, Funhand_Generate_Lanzcos.m:79-82);
* eigenvalues at X, 10 bands (Lanczos.m:18-167 as
  band_structure_woodpile_Lanczos_n60_gamma0p2.m:74-81 calls it): the FP64
  form within 1e-10 relative, the mixed form within 1e-8 relative with every
  NFSEP residual at most 1e-8.
"""
import os

import numpy as np
import pytest

import fame
from golden import make_golden as G

pytestmark = pytest.mark.gpu

N = 60
TOL = {"c128": 1e-12, "c64": 2e-5}


@pytest.fixture(scope="module")
def ops_fix():
    return np.load(G.N60_OPS_FILE)


@pytest.fixture(scope="module")
def plan(cuda, fame_lib):
    p = fame.woodpile_plan(N, [fame.fcc_point(lab) for lab in G.N60_LABELS])
    yield p
    p.close()


def dev(x, prec):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(
        device="cuda", dtype=torch.complex128 if prec == "c128" else torch.complex64)


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("inst,label", list(enumerate(G.N60_LABELS)))
def test_operators_n60_match_oracle(plan, ops_fix, prec, inst, label):
    assert np.allclose(plan.thetas[inst], ops_fix[f"{label}_theta"], rtol=0, atol=1e-15)
    Nq = N ** 3
    x, y3 = G.n60_ops_inputs(N)
    xd, yd = dev(x, prec), dev(y3, prec)
    got = {
        "Bx": plan.apply_B(xd, inst=inst),
        "Ax": plan.apply_A(xd, inst=inst),
        "Tn": plan.transform(yd, 0, inst=inst),
        "Tt": plan.transform(yd, 1, inst=inst),
        "Pr": plan.handle(0, xd[:2 * Nq], inst=inst),
        "Qr": plan.handle(1, xd[2 * Nq:], inst=inst),
        "Prs": plan.handle(2, yd, inst=inst),
        "Qrs": plan.handle(3, yd, inst=inst),
    }
    for name in G.N60_OPS:
        y = got[name].cpu().numpy().astype(np.complex128)
        err = G.digest_relerr(y, G.n60_ref(ops_fix, label, name))
        assert err < TOL[prec], (name, prec, err)


def _eig_fix():
    if not os.path.exists(G.N60_EIG_FILE):
        pytest.fail("missing fixture " + G.N60_EIG_FILE)
    return np.load(G.N60_EIG_FILE)


def test_fp64_lanczos_n60_matches_oracle(cuda, fame_lib):
    fix = _eig_fix()
    plan = fame.woodpile_plan(N, [fame.fcc_point("X")])
    assert np.allclose(plan.thetas[0], fix["theta"], rtol=0, atol=1e-15)
    r = plan.lanczos(10, tol=1e-10, maxit=10000, p=20, prec="c128", want_vectors=False)
    assert r["status"] == 0
    assert np.allclose(r["ew"], fix["ew"], rtol=1e-10, atol=0), (r["ew"], fix["ew"])
    plan.close()


def test_mixed_band_solve_n60_matches_oracle(cuda, fame_lib):
    fix = _eig_fix()
    plan = fame.woodpile_plan(N, [fame.fcc_point("X")])
    m = plan.band_solve(10, tol=1e-10, prec="c64", inner_tol=3e-12, p=26)
    assert m["status"] == 0
    assert np.allclose(m["ew"][0], fix["ew"], rtol=1e-8, atol=0), (m["ew"][0], fix["ew"])
    assert m["res"].max() <= 1e-8
    plan.close()
