"""The oracle reproduces the committed golden fixtures of the woodpile problem
(tests/golden/woodpile_golden.npz, written by tests/golden/make_golden.py):
operators to 1e-12 relative, eigenvalues to 1e-10, vertex ids exactly."""
import numpy as np
import pytest

from golden import make_golden as G

FIX = np.load(G.FILE)


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def fresh():
    return G.compute()


def test_fixture_holds_every_case():
    for n, lab in G.CASES:
        for part in ("theta", "inside", "Bx", "Ax", "Tn", "Tt"):
            assert f"n{n}_{lab}_{part}" in FIX.files
    for n, lab in G.EIG_CASES:
        assert FIX[f"n{n}_{lab}_ew"].shape == (G.BANDS,)


def test_oracle_reproduces_fixtures(fresh):
    for key in FIX.files:
        ref = FIX[key]
        got = fresh[key]
        if ref.dtype == np.uint8:
            assert np.array_equal(got, ref), key
        elif key.endswith("_ew"):
            assert np.allclose(got, ref, rtol=1e-10, atol=0), key
        elif key.endswith("_theta"):
            assert np.allclose(got, ref, rtol=1e-15, atol=0), key
        else:
            assert relerr(got, ref) < 1e-12, (key, relerr(got, ref))


def test_first_workload_fixture():
    """woodpile_n24_X.npz (written by make_golden.py --n24; ~3 minutes of
    oracle time, so not recomputed here): 10 descending eigenvalues of
    B^-1 A at the X point's Bloch angles."""
    import oracle as O

    f = np.load(G.N24_FILE)
    assert f["ew"].shape == (10,) and np.all(np.diff(f["ew"]) < 0)
    assert np.allclose(f["theta"], O.thetas_from_k(O.fcc_vertex("X")), rtol=1e-15, atol=0)


def test_fixture_geometry_is_nontrivial():
    for name in ("raster_woodpile", "raster_sphere", "raster_tetra"):
        bits = np.unpackbits(FIX[name])[:G.RASTER_N ** 3]
        assert 0 < bits.sum() < bits.size, name
