"""fame_rasterize (device vertex rasterisation) against the oracle's
isofunctions: Public/woodpile_isofun.m, the sphere isofunction of
Physical_settings_sphere.m:18 and the same-side-of-plane tetrahedron test of
Material_Locate_Isofunction.m:135-148.  The ids are integers, so the bar is
equality at every vertex."""
import numpy as np
import pytest

import fame
import oracle as O

IMAGES = [(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)]


def positions(n, A):
    return O.grid_vertices(O.Dims(n, n, n)) @ A.T


def oracle_sphere(P, A, radius, center):
    centers = np.array([np.asarray(center) + A @ np.array(m, dtype=np.float64) for m in IMAGES])
    return O.sphere_isofun(P, centers, radius)


def oracle_tetra(P, A, edge, center):
    s = edge / (2.0 * np.sqrt(2.0))
    base = s * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64)
    out = np.zeros(P.shape[0], dtype=bool)
    for m in IMAGES:
        out |= O.tetra_isofun(P, base + np.asarray(center) + A @ np.array(m, dtype=np.float64))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("n,width", [(24, 0.25), (60, 0.25), (40, 0.198)])
def test_woodpile_matches_oracle(cuda, fame_lib, n, width):
    A = fame.fcc_lattice()
    got = fame.rasterize(n, "woodpile", width, A)
    ref = O.woodpile_isofun(positions(n, A), width, 1.0)
    assert got.dtype == np.uint8 and got.shape == (n ** 3,)
    assert ref.any() and not ref.all()
    bad = np.flatnonzero(got != ref.astype(np.uint8))
    assert bad.size == 0, bad[:10]


@pytest.mark.gpu
@pytest.mark.parametrize("n,radius,center", [(40, 0.25, (0.0, 0.0, 0.0)), (60, 0.25, (0.0, 0.0, 0.0)),
                                             (48, 0.2, (0.5, 0.5, 0.5))])
def test_sphere_matches_oracle(cuda, fame_lib, n, radius, center):
    A = fame.fcc_lattice()
    got = fame.rasterize(n, "sphere", radius, A, center=center)
    ref = oracle_sphere(positions(n, A), A, radius, center)
    assert ref.any()
    bad = np.flatnonzero(got != ref.astype(np.uint8))
    assert bad.size == 0, bad[:10]


@pytest.mark.gpu
@pytest.mark.parametrize("n,edge", [(40, 0.5), (60, 0.5), (32, 0.7)])
def test_tetra_matches_oracle(cuda, fame_lib, n, edge):
    A = fame.fcc_lattice()
    got = fame.rasterize(n, "tetra", edge, A)
    ref = oracle_tetra(positions(n, A), A, edge, (0.0, 0.0, 0.0))
    assert ref.any()
    bad = np.flatnonzero(got != ref.astype(np.uint8))
    assert bad.size == 0, bad[:10]


@pytest.mark.gpu
def test_paint_union_and_device_output(cuda, fame_lib):
    """Two inclusions painted into one id array (the union of
    Material_Locate_Isofunction.m:22-25), on the device and through host
    memory."""
    import torch

    n = 32
    A = fame.fcc_lattice()
    P = positions(n, A)
    wood = O.woodpile_isofun(P, 0.25, 1.0)
    sph = oracle_sphere(P, A, 0.15, (0.25, 0.25, 0.25))
    ref = np.where(sph, 2, wood.astype(np.uint8)).astype(np.uint8)
    d = fame.rasterize(n, "woodpile", 0.25, A, device=True)
    assert isinstance(d, torch.Tensor) and d.is_cuda
    fame.rasterize(n, "sphere", 0.15, A, center=(0.25, 0.25, 0.25), phase_id=2, phase=d)
    assert np.array_equal(d.cpu().numpy(), ref)
    h = fame.rasterize(n, "woodpile", 0.25, A)
    h = fame.rasterize(n, "sphere", 0.15, A, center=(0.25, 0.25, 0.25), phase_id=2, phase=h)
    assert np.array_equal(h, ref)


@pytest.mark.gpu
def test_plan_from_device_phases_matches_oracle_problem(cuda, fame_lib):
    """woodpile_plan builds its phase ids with the device rasteriser; its fncB
    equals the oracle's on the oracle's own geometry."""
    import torch

    n = 8
    kvec = fame.fcc_point("X")
    plan = fame.woodpile_plan(n, [kvec])
    P = O.build_problem(n, wave_vec=kvec)
    x = np.random.default_rng(3).standard_normal(4 * n ** 3) + 1j * np.random.default_rng(4).standard_normal(4 * n ** 3)
    y = plan.apply_B(torch.as_tensor(x, device="cuda")).cpu().numpy()
    yo = O.fncB(x, P.fnc, P.mat)
    assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)


def test_bad_arguments_rejected_on_host(fame_lib):
    """Argument checks run before any device work (no GPU needed)."""
    import ctypes as C

    from fame import _lib as L

    A = np.ascontiguousarray(fame.fcc_lattice())
    out = np.zeros(8, dtype=np.uint8)
    pd = C.POINTER(C.c_double)
    for shape, params, n in [(7, [0.25, 1.0], 2), (0, [-0.25, 1.0], 2), (1, [0.0, 0, 0, 0], 2),
                             (0, [0.25, 1.0], 0), (2, [np.nan, 0, 0, 0], 2)]:
        p = np.asarray(params + [0.0] * (4 - len(params)), dtype=np.float64)
        rc = fame_lib.fame_rasterize(n, A.ctypes.data_as(pd), shape, p.ctypes.data_as(pd), 1,
                                     C.c_void_p(out.ctypes.data), L.FAME_HOST_PTR)
        assert rc == L.FAME_ERR_BAD_ARG
        assert b"fame_rasterize" in fame_lib.fame_last_error(None)
    with pytest.raises(fame.FameError):
        fame.rasterize(2, "woodpile", -1.0)
    with pytest.raises(ValueError, match="unknown shape"):
        fame.rasterize(2, "cube", 0.25)
    with pytest.raises(ValueError, match="n\\^3"):
        fame.rasterize(2, "woodpile", 0.25, phase=np.zeros(5, dtype=np.uint8))
