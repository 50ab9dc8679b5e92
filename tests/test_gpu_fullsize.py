"""Size-independent properties of the operators at the benchmark's full size
(n = 60; the operators' values there are held to the oracle by
test_gpu_n60.py): the S-phased DFT is unitary and its 'transpose' inverts
it, Prs / Qrs invert Pr / Qr, fncA and fncB are Hermitian, fncB is positive
definite and linear, complex64 agrees with complex128, and fncinvB inverts
fncB."""
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


def test_empty_and_bad_batches(plan):
    """An empty batch is a no-op; a negative count, missing vectors and an
    instance index outside the plan are rejected before any device work."""
    from fame import _lib as L

    lib = fame.load()
    h = plan.raw
    for fn in (lib.fame_apply_A, lib.fame_apply_B):
        assert fn(h, L.FAME_C128, None, None, 0, None, 0) == L.FAME_OK
        assert fn(h, L.FAME_C128, None, None, -1, None, 0) == L.FAME_ERR_BAD_ARG
        assert fn(h, L.FAME_C128, None, None, 1, None, 0) == L.FAME_ERR_BAD_ARG
    assert lib.fame_apply_Binv(h, L.FAME_C128, None, None, 0, None, 1e-10, 100, None, None, 0) == L.FAME_OK
    x = rand(4 * N ** 3, 1, 8)
    y = torch.empty_like(x)
    import ctypes as C

    bad = (C.c_int * 1)(5)
    rc = lib.fame_apply_B(h, L.FAME_C128, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), 1, bad, 0)
    assert rc == L.FAME_ERR_BAD_ARG
    assert b"instance" in lib.fame_last_error(h)


def test_largest_compiled_grid(cuda, fame_lib):
    """n = 64, the largest compiled size: DFT round trip, Hermitian fncB and
    complex64 against complex128."""
    n = 64
    p = fame.woodpile_plan(n, [fame.fcc_point("W")])
    try:
        x3 = rand(3 * n ** 3, 1, 9)
        assert rel(p.transform(p.transform(x3, 0), 1), x3) < 1e-13
        x = rand(4 * n ** 3, 1, 10)
        y = rand(4 * n ** 3, 1, 11)
        bx, by = p.apply_B(x), p.apply_B(y)
        s1, s2 = torch.vdot(y[0], bx[0]), torch.vdot(x[0], by[0]).conj()
        assert abs(complex(s1 - s2)) < 1e-12 * float(torch.linalg.norm(y[0]) * torch.linalg.norm(bx[0]))
        assert rel(p.apply_B(x.to(torch.complex64)).to(torch.complex128), bx) < 5e-5
    finally:
        p.close()
