"""Host logic of the product (no GPU needed): geometry, constitutive blocks,
k-paths, and the C ABI's host-only material helper."""
import numpy as np
import pytest

import fame
import oracle as O


@pytest.mark.parametrize("n", [12, 24, 60])
def test_woodpile_rasterisation_matches_oracle(n):
    A = fame.fcc_lattice()
    prod = fame.woodpile_inside(fame.vertex_positions(n, A), 0.25)
    ref = O.woodpile_isofun(O.grid_vertices(O.Dims(n, n, n)) @ A.T, 0.25, 1.0)
    assert np.array_equal(prod, ref)
    assert 0.1 < prod.mean() < 0.6


def test_bloch_angles():
    th = fame.bloch_angles(fame.fcc_point("X"))
    assert np.allclose(th, [np.pi, 0.0, np.pi])
    assert np.allclose(fame.bloch_angles([0, 0, 0]), O.thetas_from_k([0, 0, 0]))


def test_material_blocks_match_oracle(fame_lib):
    A = fame.fcc_lattice()
    rng = np.random.default_rng(3)
    for _ in range(4):
        eps = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3)) + 4 * np.eye(3)
        mu = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3)) + 4 * np.eye(3)
        xi = 0.3 * (rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3)))
        zeta = 0.3 * (rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3)))
        got = fame.covariant_blocks(fame.constitutive(eps, mu, xi, zeta), A)
        ref = O.material_blocks(O.Phase(eps, mu, xi, zeta), A)
        assert np.allclose(got, np.concatenate([b.ravel() for b in ref]), rtol=1e-13, atol=1e-13)
    with pytest.raises(fame.FameError, match="singular"):
        fame.covariant_blocks(np.zeros((6, 6)), A)


def test_band_path_40():
    k = fame.band_path(npts=40)
    assert k.shape == (40, 3)
    assert np.allclose(k[0], 0.0)
    for lab in "XULWK":
        assert np.min(np.linalg.norm(k - fame.fcc_point(lab), axis=1)) < 1e-12
    assert np.allclose(k[-1], fame.fcc_point("X"))


def test_reference_path_construction():
    # Physical_settings_woodpile.m:165-182 with 'XULGXWK', part_num = 10: 6 segments,
    # 9 new points each plus the final end point
    k = fame.reference_path("XULGXWK", 10)
    assert k.shape == (55, 3)
    assert np.allclose(k[0], fame.fcc_point("X")) and np.allclose(k[-1], fame.fcc_point("K"))
    assert np.allclose(k[9], fame.fcc_point("U"))


def test_sphere_periodic_images():
    A = fame.fcc_lattice()
    P = fame.vertex_positions(12, A)
    m = fame.sphere_inside(P, 0.25, A)
    frac = m.mean()
    vol = 4 / 3 * np.pi * 0.25 ** 3 / abs(np.linalg.det(A))
    assert abs(frac - vol) < 0.05


def test_tetra_inside_matches_oracle_isofun():
    """fame.tetra_inside (periodic images) against the oracle's four
    half-space test (Material_Locate_Isofunction.m) applied to each image."""
    import oracle as O
    A = fame.fcc_lattice()
    P = fame.vertex_positions(12, A)
    edge = 0.5
    s = edge / (2.0 * np.sqrt(2.0))
    base = s * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64)
    ref = np.zeros(P.shape[0], dtype=bool)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                ref |= O.tetra_isofun(P, base + A @ np.array([i, j, k], dtype=np.float64))
    got = fame.tetra_inside(P, edge, A)
    assert got.sum() > 0
    assert np.array_equal(got, ref)


def test_ibz_points_in_wedge():
    import fame.batch as FB
    k = FB.ibz_kpoints(200, seed=1) / (2 * np.pi)
    assert np.all(k[:, 2] <= k[:, 0] + 1e-15) and np.all(k[:, 0] <= k[:, 1] + 1e-15)
    assert np.all(k.sum(axis=1) <= 1.5 + 1e-12) and np.all(k <= 1.0)
    # the high-symmetry points bounding the wedge, in fame.fcc_point's orientation
    for lab in "GXLWKU":
        q = fame.fcc_point(lab) / (2 * np.pi)
        assert q[2] <= q[0] + 1e-12 <= q[1] + 2e-12 and q.sum() <= 1.5 + 1e-12
