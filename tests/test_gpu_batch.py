"""Uneven-grid batch (fame.batch): plans of several grid sizes solved
concurrently on their own streams give the same eigenvalues as solving each
instance alone, and the autotuner's choice leaves fncB unchanged."""
import numpy as np
import pytest
import torch

import fame
import fame.batch as FB

pytestmark = pytest.mark.gpu


def test_uneven_concurrent_matches_single_instances(cuda, fame_lib):
    groups = FB.uneven_workload(seed=3, sizes=(8, 12), per_size=3, bands=(3, 5))
    res, wall = FB.solve_uneven(groups, prec="c128", tol=1e-10, concurrent=True)
    seq, _ = FB.solve_uneven(groups, prec="c128", tol=1e-10, concurrent=False, autotune=False)
    for g, r, s in zip(groups, res, seq):
        assert r["status"] == 0 and s["status"] == 0
        for i in range(len(g["kvecs"])):
            assert len(r["omega"][i]) == g["bands"][i]
            assert np.allclose(r["omega"][i], s["omega"][i], rtol=1e-10)
        # instance 0 on its own plan
        plan = fame.woodpile_plan(g["n"], g["kvecs"][:1], gamma=float(g["gammas"][0]))
        k = int(g["bands"][0])
        one = plan.lanczos(k, tol=1e-10, prec="c128", p=max(2 * k, 20), want_vectors=False)
        assert np.allclose(np.sort(one["omega"]), r["omega"][0], rtol=1e-9)


@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_autotuned_fncB_unchanged(cuda, fame_lib, dtype):
    """Sub-batch widths never change a result; within one stencil form
    (single pass, or two kernels at any block size) results are bit-identical,
    and the two forms agree to rounding (their vertex products are summed in
    different orders)."""
    plan = fame.woodpile_plan(12, fame.band_path(npts=40)[:5])
    rng = np.random.default_rng(0)
    x = rng.standard_normal((5, 4 * 12 ** 3)) + 1j * rng.standard_normal((5, 4 * 12 ** 3))
    xt = torch.as_tensor(x).to(torch.complex64 if dtype == "c64" else torch.complex128).cuda()
    pr = 1 if dtype == "c64" else 0
    lib = fame.load()
    t = plan.autotune(nvec=5, prec=dtype)
    assert t["chunk"] in (0, 1, 2, 3, 4) and t["stencil_tpb"] in (0, 128, 256, 512) and t["us"] > 0
    ref = {}
    for form, tpbs in (("sweep", (0,)), ("two-kernel", (128, 512))):
        for chunk in (1, 2, 0):
            for tpb in tpbs:
                assert lib.fame_set_tune(plan.raw, pr, 5, chunk, tpb) == 0
                y = plan.apply_B(xt)
                if form not in ref:
                    ref[form] = y
                assert torch.equal(y, ref[form]), (form, chunk, tpb)
    tol = 1e-6 if dtype == "c64" else 1e-14
    d = torch.linalg.norm(ref["sweep"] - ref["two-kernel"]) / torch.linalg.norm(ref["two-kernel"])
    assert float(d) < tol


@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_plane_lanes_give_the_same_fncB(cuda, fame_lib, dtype):
    """The plane kernels' split of each FFT pencil (threads per pencil: the
    prime-factor splits 60 = 3*20, 4*15, 5*12 compiled at n = 60, or one
    thread per pencil) changes how the DFTs are evaluated, not the operator:
    every lane count agrees with the default to rounding, an unknown count
    falls back to the default bit for bit, and the autotuner reports a
    compiled choice."""
    n = 60
    plan = fame.woodpile_plan(n, fame.band_path(npts=40)[:2])
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 4 * n ** 3)) + 1j * rng.standard_normal((2, 4 * n ** 3))
    xt = torch.as_tensor(x).to(torch.complex64 if dtype == "c64" else torch.complex128).cuda()
    plan.set_tune(dtype, 2, 0, 0 if dtype == "c64" else 256, -1)
    ref = plan.apply_B(xt)
    assert plan.get_tune(dtype, 2)["lanes"] == -1
    tol = 2e-6 if dtype == "c64" else 1e-13
    for lanes in (0, 3, 4, 5):
        plan.set_tune(dtype, 2, 0, 0 if dtype == "c64" else 256, lanes)
        assert plan.get_tune(dtype, 2)["lanes"] == lanes
        y = plan.apply_B(xt)
        d = float(torch.linalg.norm(y - ref) / torch.linalg.norm(ref))
        assert d < tol, (lanes, d)
        if lanes == 3:
            assert torch.equal(y, ref)  # 3 is the default at n = 60
    plan.set_tune(dtype, 2, 0, 0 if dtype == "c64" else 256, 7)  # not compiled: the default
    assert torch.equal(plan.apply_B(xt), ref)
    t = plan.autotune(nvec=2, prec=dtype)
    assert t["lanes"] in (-1, 0, 3, 4, 5)
    plan.close()
