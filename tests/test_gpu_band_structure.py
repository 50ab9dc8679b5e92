"""fame.band_structure: the band-structure driver of
band_structure_woodpile_Lanczos_n60_gamma0p2.m:39-123 with its result arrays
(Freq_mtx, iter_records, time_compute_eigs, res_NFSEP, res_ORGSEP) written to
an .npz file.  Batched frequencies equal the oracle's per-k Lanczos."""
import numpy as np
import pytest

import fame
import oracle as O
from fame.band_structure import band_structure

pytestmark = pytest.mark.gpu


def test_band_structure_arrays_and_npz(cuda, fame_lib, tmp_path):
    n, bands = 8, 4
    kv = fame.band_path(labels=("X", "W", "L"), npts=5)
    out = tmp_path / "bands.npz"
    r = band_structure(n, kv, bands, batch=2, prec="c128", tol=1e-10, out=str(out))
    f = np.load(out)
    assert f["Freq_mtx"].shape == (bands, 5)
    assert np.array_equal(f["Freq_mtx"], r["Freq_mtx"])
    assert np.array_equal(f["wave_vec_array"], kv.T)
    assert (f["iter_records"] > 0).all() and (f["time_compute_eigs"] > 0).all()
    assert (f["status"] == 0).all()
    assert f["res_NFSEP"].max() <= 1e-8
    assert np.isfinite(f["res_ORGSEP"]).all()
    # per-k against the oracle's Lanczos on the oracle's own problem
    for i in (0, 3):
        P = O.build_problem(n, wave_vec=kv[i])
        v0 = np.ones(4 * n ** 3, dtype=np.complex128)
        v0 = v0 / np.sqrt(abs(np.vdot(v0, P.B(v0))))
        _, ew, _ = O.lanczos(P.A, P.B, lambda x: O.fncinvB(x, P.B), 4 * n ** 3, bands, 1e-10, 1000, 2 * bands, v0)
        om = np.sort(1.0 / np.asarray(ew))
        assert np.allclose(r["Freq_mtx"][:, i], om, rtol=1e-9)


def test_band_structure_mixed_matches_fp64(cuda, fame_lib):
    n, bands = 8, 4
    kv = fame.band_path(labels=("X", "U"), npts=4)
    a = band_structure(n, kv, bands, batch=4, prec="c128", tol=1e-10, orgsep=False)
    b = band_structure(n, kv, bands, batch=4, prec="c64", tol=1e-10, orgsep=False)
    assert np.allclose(a["Freq_mtx"], b["Freq_mtx"], rtol=1e-8)
    assert b["res_NFSEP"].max() <= 1e-8
    assert np.isnan(b["res_ORGSEP"]).all()
