"""Size-independent properties of the operators at the benchmark's full size
(n = 60, where the oracle's sparse assembly is too slow to run in a test):
the S-phased DFT is unitary and its 'transpose' inverts it, Prs / Qrs invert
Pr / Qr, fncA and fncB are Hermitian, fncB is positive definite and linear,
complex64 agrees with complex128, and fncinvB inverts fncB."""
import pytest
import torch

import fame

pytestmark = pytest.mark.gpu

N = 60


@pytest.fixture(scope="module")
def plan(cuda, fame_lib):
    p = fame.woodpile_plan(N, [fame.fcc_point("X"), fame.fcc_point("L")])
    yield p
    p.close()


def rand(length, nvec, seed, dtype=torch.complex128):
    g = torch.Generator(device="cuda").manual_seed(seed)
    re = torch.randn(nvec, length, generator=g, device="cuda", dtype=torch.float64)
    im = torch.randn(nvec, length, generator=g, device="cuda", dtype=torch.float64)
    return torch.complex(re, im).to(dtype)


def rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.parametrize("prec,tol", [("c128", 1e-13), ("c64", 5e-6)])
def test_transform_unitary_and_inverse(plan, prec, tol):
    dt = torch.complex128 if prec == "c128" else torch.complex64
    x = rand(3 * N ** 3, 2, 1, dt)
    y = plan.transform(x, 0)
    z = plan.transform(y, 1)
    assert rel(z, x) < tol
    nx = torch.linalg.norm(x, dim=1).double()
    ny = torch.linalg.norm(y, dim=1).double()
    assert float(torch.max(torch.abs(ny / nx - 1))) < tol


@pytest.mark.parametrize("prec,tol", [("c128", 1e-13), ("c64", 5e-6)])
def test_handles_are_isometries(plan, prec, tol):
    dt = torch.complex128 if prec == "c128" else torch.complex64
    a = rand(2 * N ** 3, 2, 2, dt)
    assert rel(plan.handle(2, plan.handle(0, a)), a) < tol  # Prs(Pr a) = a
    assert rel(plan.handle(3, plan.handle(1, a)), a) < tol  # Qrs(Qr a) = a


def test_fncA_fncB_hermitian_and_positive(plan):
    L = 4 * N ** 3
    x = rand(L, 2, 3)
    y = rand(L, 2, 4)
    bx, by = plan.apply_B(x), plan.apply_B(y)
    ax, ay = plan.apply_A(x), plan.apply_A(y)
    for v in range(2):
        s1 = torch.vdot(y[v], bx[v])
        s2 = torch.vdot(x[v], by[v]).conj()
        scale = float(torch.linalg.norm(y[v]) * torch.linalg.norm(bx[v]))
        assert abs(complex(s1 - s2)) < 1e-12 * scale
        q = torch.vdot(x[v], bx[v])
        assert float(q.real) > 0 and abs(float(q.imag)) < 1e-12 * float(q.real)
        t1 = torch.vdot(y[v], ax[v])
        t2 = torch.vdot(x[v], ay[v]).conj()
        assert abs(complex(t1 - t2)) < 1e-12 * float(torch.linalg.norm(y[v]) * torch.linalg.norm(ax[v]))


def test_fncB_linear_and_c64_matches_c128(plan):
    L = 4 * N ** 3
    x = rand(L, 2, 5)
    y = rand(L, 2, 6)
    a, b = 0.3 - 1.7j, 2.1 + 0.4j
    lhs = plan.apply_B(a * x + b * y)
    rhs = a * plan.apply_B(x) + b * plan.apply_B(y)
    assert rel(lhs, rhs) < 1e-13
    b64 = plan.apply_B(x)
    b32 = plan.apply_B(x.to(torch.complex64)).to(torch.complex128)
    assert rel(b32, b64) < 5e-5


def test_fncinvB_inverts_fncB(plan):
    L = 4 * N ** 3
    b = rand(L, 2, 7)
    x = plan.apply_Binv(b, tol=1e-10, maxit=10000, raise_on_noconv=True)
    x = x[0] if isinstance(x, tuple) else x
    assert rel(plan.apply_B(x), b) < 5e-10
