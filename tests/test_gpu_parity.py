"""CUDA library vs the CPU oracle on the same seeded inputs (complex128 to
1e-12, complex64 to 2e-5 relative).  Sizes are small enough for the oracle's
sparse assembly to finish in seconds."""
import numpy as np
import pytest

import fame
import oracle as O
from problems import Pair, relerr

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 2e-5}


def _dev(x, prec):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(
        device="cuda", dtype=torch.complex128 if prec == "c128" else torch.complex64)


@pytest.mark.parametrize("n", [4, 6, 8, 12])
@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("hermitian", [True, False])
def test_fncB(cuda, fame_lib, n, prec, hermitian):
    P = Pair(n, nk=2, seed=n, hermitian=hermitian)
    L = 4 * P.Nq
    x = P.vec(L, 3)
    inst = [1, 0, 1]
    y = P.plan.apply_B(_dev(x, prec), inst=inst).cpu().numpy()
    for v in range(3):
        svd, fnc, mat = P.ref(inst[v])
        yr = O.fncB(x[v], fnc, mat)
        assert relerr(y[v], yr) < TOL[prec], (v, relerr(y[v], yr))


@pytest.mark.parametrize("n", [6, 10])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_fncA(cuda, fame_lib, n, prec):
    P = Pair(n, nk=2, seed=3)
    x = P.vec(4 * P.Nq, 2)
    y = P.plan.apply_A(_dev(x, prec)).cpu().numpy()
    for v in range(2):
        svd, _, _ = P.ref(v)
        assert relerr(y[v], O.fncA(x[v], svd.Sigma_r)) < TOL[prec]


@pytest.mark.parametrize("n", [4, 8, 12])
@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("trans", ["notranspose", "transpose"])
def test_mtxvecmul_fft(cuda, fame_lib, n, prec, trans):
    P = Pair(n, nk=2, seed=5)
    x = P.vec(3 * P.Nq, 2)
    y = fame.MtxVecMul_FFT(_dev(x, prec), P.plan, trans).cpu().numpy()
    for v in range(2):
        svd, _, _ = P.ref(v)
        yr = O.mtxvecmul_fft(x[v], svd.dims, trans, svd.S, svd.D)
        assert relerr(y[v], yr) < TOL[prec]


@pytest.mark.parametrize("which", ["Pr", "Qr", "Prs", "Qrs"])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_handles(cuda, fame_lib, which, prec):
    P = Pair(6, nk=2, seed=7)
    code = {"Pr": 0, "Qr": 1, "Prs": 2, "Qrs": 3}[which]
    L = (2 if code < 2 else 3) * P.Nq
    x = P.vec(L, 2)
    y = P.plan.handle(code, _dev(x, prec)).cpu().numpy()
    for v in range(2):
        _, fnc, _ = P.ref(v)
        yr = getattr(fnc, which)(x[v])
        assert relerr(y[v], yr) < TOL[prec]


@pytest.mark.parametrize("hermitian", [True, False])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_material_operator(cuda, fame_lib, hermitian, prec):
    P = Pair(6, nk=2, seed=11, hermitian=hermitian, nphase=3)
    N = P.Nq
    x = P.vec(6 * N, 2)
    y = P.plan.material(_dev(x, prec)).cpu().numpy()
    for v in range(2):
        _, _, mat = P.ref(v)
        u, w = x[v][:3 * N], x[v][3 * N:]
        yr = np.concatenate([mat.M_int @ u + mat.J_intH @ w, mat.J_int @ u + mat.N_int @ w])
        assert relerr(y[v], yr) < TOL[prec]


def test_host_pointer_path(cuda, fame_lib):
    P = Pair(6, nk=1, seed=2)
    x = P.vec(4 * P.Nq, 2)
    y_host = P.plan.apply_B(x)                       # NumPy in, NumPy out (staged)
    y_dev = P.plan.apply_B(_dev(x, "c128")).cpu().numpy()
    assert relerr(y_host, y_dev) < 1e-15


def test_fncinvB_pcg(cuda, fame_lib):
    P = Pair(8, nk=2, seed=13)
    x = P.vec(4 * P.Nq, 2)
    xd = _dev(x, "c128")
    y, its, rr = P.plan.apply_Binv(xd, tol=1e-11, maxit=5000)
    back = P.plan.apply_B(y).cpu().numpy()
    for v in range(2):
        assert relerr(back[v], x[v]) < 2e-11
        assert rr[v] < 1e-11 and its[v] > 0
        _, fnc, mat = P.ref(v)
        ref, flag, relres, it = O.pcg_matlab(lambda z: O.fncB(z, fnc, mat), x[v], 1e-11, 5000)
        assert flag == 0
        assert relerr(y.cpu().numpy()[v], ref) < 1e-9


def test_fncinvB_c64(cuda, fame_lib):
    P = Pair(8, nk=1, seed=17)
    x = P.vec(4 * P.Nq)
    y, its, rr = P.plan.apply_Binv(_dev(x, "c64"), tol=1e-5, maxit=2000)
    back = P.plan.apply_B(_dev(y.cpu().numpy(), "c128")).cpu().numpy()
    assert relerr(back, x) < 3e-5


def test_fncinvB_reports_breakdown_and_nan(cuda, fame_lib):
    # Failure detection on the host: an indefinite B (strong J coupling) makes CG
    # break down (p'Bp <= 0) and a NaN right-hand side yields FAME_ERR_NAN; both
    # come back as status codes, the context stays usable.
    n = 6
    I3 = np.eye(3).ravel()
    tens = np.concatenate([I3, I3, 3.0 * I3]).astype(complex)[None, :]
    plan = fame.Plan(n, [[0.4, -0.2, 1.1]], np.zeros(n ** 3, np.uint8), tens)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(4 * n ** 3) + 1j * rng.standard_normal(4 * n ** 3)
    with pytest.raises(fame.FameError) as e:
        plan.apply_Binv(_dev(x, "c128"), tol=1e-10, maxit=500, raise_on_noconv=True)
    assert e.value.code == 4
    P = Pair(6, nk=1, seed=3)
    xn = P.vec(4 * P.Nq)
    xn[5] = np.nan
    with pytest.raises(fame.FameError) as e:
        P.plan.apply_Binv(_dev(xn, "c128"), tol=1e-10, maxit=50, raise_on_noconv=True)
    assert e.value.code in (4, 5)
    y = P.plan.apply_B(_dev(P.vec(4 * P.Nq), "c128"))  # still usable
    assert np.isfinite(y.cpu().numpy()).all()


def test_errors(cuda, fame_lib):
    import torch

    with pytest.raises(fame.FameError) as e:
        fame.Plan(7, [[0.1, 0.2, 0.3]], np.zeros(343, np.uint8), np.zeros((1, 27), complex))
    assert e.value.code == 6  # unsupported grid size
    with pytest.raises(fame.FameError) as e:
        fame.Plan(6, [[0.0, 0.0, 0.0]], np.zeros(216, np.uint8), np.zeros((1, 27), complex))
    assert e.value.code == 7  # singular at Gamma without the 1e-4 shift
    with pytest.raises(fame.FameError) as e:
        fame.Plan(6, [[0.1, 0.2, 0.3]], np.full(216, 3, np.uint8), np.zeros((2, 27), complex))
    assert e.value.code == 1  # phase id out of range
    P = Pair(6, nk=2, seed=1)
    with pytest.raises(fame.FameError) as e:
        P.plan.apply_B(_dev(P.vec(4 * P.Nq, 2), "c128"), inst=[0, 5])
    assert e.value.code == 1
    empty = torch.zeros((0, 4 * P.Nq), dtype=torch.complex128, device="cuda")
    assert P.plan.apply_B(empty).shape == (0, 4 * P.Nq)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_cg_graph_replay_matches_direct_launches(cuda, fame_lib, prec):
    """The CG loop replayed from one graph launch (device-side loop
    condition), blocks of CG iterations replayed from captured CUDA graphs,
    and every kernel launched directly give the same iterates (same kernels,
    same order)."""
    pr = Pair(8, nk=2, seed=21)
    rng = np.random.default_rng(5)
    b = rng.standard_normal((3, 4 * pr.Nq)) + 1j * rng.standard_normal((3, 4 * pr.Nq))
    import torch
    bt = torch.as_tensor(b).to(torch.complex128 if prec == "c128" else torch.complex64).cuda()
    tol = 1e-10 if prec == "c128" else 1e-5
    out = {}
    for g in (2, 1, 0):
        pr.plan.set_option("graph", g)
        y, its, rr = pr.plan.apply_Binv(bt, tol=tol, maxit=2000)
        y2, its2, _ = pr.plan.apply_Binv(bt, tol=tol, maxit=2000)
        assert torch.equal(y, y2) and np.array_equal(its, its2)  # second call replays the cached graph
        out[g] = (y.cpu().numpy(), its.copy(), rr.copy())
    pr.plan.set_option("graph", 2)
    for g in (2, 1):
        assert np.array_equal(out[g][1], out[0][1])
        assert np.array_equal(out[g][0], out[0][0])
