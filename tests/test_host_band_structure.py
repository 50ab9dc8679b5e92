"""Host logic of fame.band_structure (batching, result arrays, .npz file)
with a stand-in plan: no GPU."""
import numpy as np

import fame.band_structure as BS


class FakePlan:
    made = []

    def __init__(self, n, kv, **kw):
        self.kv = np.atleast_2d(kv)
        self.nk = self.kv.shape[0]
        self.tuned = None
        self.closed = False
        FakePlan.made.append(self)

    def autotune(self, nvec=None, prec="c64"):
        self.tuned = ("auto", nvec)
        return {"chunk": 2, "stencil_tpb": 128, "lanes": 4}

    def set_tune(self, prec, nvec, chunk, tpb, lanes=-1):
        self.tuned = ("set", nvec, chunk, tpb, lanes)

    def autotune_mixed(self, nvec=None):
        return {"c64": self.autotune(nvec=nvec, prec="c64"), "c128ds": self.autotune(nvec=nvec, prec="c128ds")}

    def set_tune_mixed(self, nvec, tunes):
        for prec, t in tunes.items():
            self.set_tune(prec, nvec, t["chunk"], t["stencil_tpb"], t.get("lanes", -1))

    def band_solve(self, k, tol, p, prec, inner_tol, want_vectors):
        key = self.kv[:, 0][:, None]  # first wave-vector component identifies the k-point
        om = key + np.arange(k)[None, :] / 100.0
        ev = np.arange(self.nk * k * 3, dtype=np.float64).reshape(self.nk, k, 3) if want_vectors else None
        stats = np.tile(np.array([[11, 2, 33, 44]]), (self.nk, 1))
        return dict(ew=1.0 / om, omega=om, res=om * 1e-12, stats=stats, status=0, ev=ev)

    def restore(self, ev, omega, inst=None, want_fields=True):
        assert ev.shape[0] == len(omega) == len(inst)
        return dict(res_orgsep=np.asarray(omega) * 1e-9)

    def sync(self):
        pass

    def close(self):
        self.closed = True


def test_batches_map_back_to_path_order(monkeypatch, tmp_path):
    FakePlan.made = []
    monkeypatch.setattr(BS, "woodpile_plan", FakePlan)
    kv = np.stack([np.array([float(i + 1), 0.0, 0.0]) for i in range(7)])
    out = tmp_path / "b.npz"
    r = BS.band_structure(12, kv, bands=4, batch=3, prec="c64", out=str(out))
    assert [p.nk for p in FakePlan.made] == [3, 3, 1]
    assert all(p.closed for p in FakePlan.made)
    assert FakePlan.made[0].tuned == ("auto", 3)
    assert FakePlan.made[1].tuned == ("set", 3, 2, 128, 4)
    expect = (np.arange(7) + 1.0)[None, :] + np.arange(4)[:, None] / 100.0
    assert np.allclose(r["Freq_mtx"], expect)
    assert np.allclose(r["res_ORGSEP"], expect * 1e-9)
    assert np.allclose(r["res_NFSEP"], expect * 1e-12)
    assert (r["iter_records"] == 11).all() and (r["cg_iterations"] == 44).all()
    assert (r["time_compute_eigs"] > 0).all()
    f = np.load(out)
    for key in ("Freq_mtx", "iter_records", "time_compute_eigs", "res_NFSEP", "res_ORGSEP", "wave_vec_array"):
        assert np.array_equal(f[key], r[key])
    assert f["wave_vec_array"].shape == (3, 7)


def test_fp64_form_skips_autotune_and_orgsep(monkeypatch):
    FakePlan.made = []
    monkeypatch.setattr(BS, "woodpile_plan", FakePlan)
    kv = np.stack([np.array([float(i + 1), 0.0, 0.0]) for i in range(4)])
    r = BS.band_structure(12, kv, bands=2, batch=4, prec="c128", orgsep=False)
    assert FakePlan.made[0].tuned is None
    assert np.isnan(r["res_ORGSEP"]).all()
    assert r["Freq_mtx"].shape == (2, 4)


def test_concurrent_batches_fill_the_same_arrays(monkeypatch):
    """Batches solved on concurrent host threads land in the same places as
    one after another; the first batch is tuned alone and the others get its
    setting."""
    monkeypatch.setattr(BS, "woodpile_plan", FakePlan)
    kv = np.stack([np.array([float(i + 1), 0.0, 0.0]) for i in range(11)])
    FakePlan.made = []
    seq = BS.band_structure(12, kv, bands=3, batch=2, prec="c64", concurrent=1)
    FakePlan.made = []
    con = BS.band_structure(12, kv, bands=3, batch=2, prec="c64", concurrent=3)
    assert sorted(p.nk for p in FakePlan.made) == [1, 2, 2, 2, 2, 2]
    assert all(p.closed for p in FakePlan.made)
    # one autotune per batch width (2 and the last batch's 1), the rest installed
    assert sum(1 for p in FakePlan.made if p.tuned and p.tuned[0] == "auto") == 2
    assert sum(1 for p in FakePlan.made if p.tuned and p.tuned[0] == "set") == 4
    for key in ("Freq_mtx", "res_NFSEP", "res_ORGSEP", "iter_records", "cg_iterations", "status"):
        assert np.array_equal(seq[key], con[key]), key
