"""The FP64 refinement sweep of the mixed form (FAME_OPT_REFINE): one block
inverse-iteration step Y = B^-1 A X with FP64 Rayleigh-Ritz on [X Y] per
k-point.  The refined eigenvalues must stay those of the FP64 form
(Lanczos.m:18-167, 1e-9 relative), the NFSEP residuals
(EvaluteError_Chiral_no_inv.m:20) must not grow, the residuals before the
sweep are reported, and the per-instance statistics count each instance's
own B applies."""
import numpy as np
import pytest

import fame

pytestmark = pytest.mark.gpu


def test_refinement_keeps_eigenvalues_and_lowers_residuals(cuda, fame_lib):
    n, k = 12, 6
    kv = [fame.fcc_point("X"), fame.fcc_point("L"), fame.fcc_point("W")]
    plan = fame.woodpile_plan(n, kv)
    ref = plan.band_solve(k, tol=1e-11, prec="c128", inner_tol=1e-13, p=2 * k)
    assert ref["status"] == 0 and ref["res_before"] is None  # no sweep in the FP64 form
    plan.set_option("refine", 0)
    raw = plan.band_solve(k, tol=1e-8, prec="c64", inner_tol=1e-10, p=2 * k + 4, want_vectors=True)
    plan.set_option("refine", 1)
    ref_m = plan.band_solve(k, tol=1e-8, prec="c64", inner_tol=1e-10, p=2 * k + 4, want_vectors=True)
    assert raw["status"] == 0 and ref_m["status"] == 0
    assert raw["res_before"] is None
    rb = ref_m["res_before"]
    assert rb is not None and rb.shape == ref_m["res"].shape
    # before the sweep: the unrefined solve's residuals
    assert np.allclose(rb, raw["res"], rtol=1e-6, atol=1e-14)
    assert ref_m["res"].max() <= rb.max()
    assert np.allclose(ref_m["ew"], ref["ew"], rtol=1e-9, atol=0), (ref_m["ew"], ref["ew"])
    # refined vectors are B-normalised eigenvectors: ||B x - omega A x|| as reported
    ev = ref_m["ev"]
    for a in range(len(kv)):
        bx = plan.apply_B(ev[a], inst=a).cpu().numpy()
        ax = plan.apply_A(ev[a], inst=a).cpu().numpy()
        x = ev[a].cpu().numpy()
        for i in range(k):
            assert abs(np.vdot(x[i], bx[i]).real - 1.0) < 1e-9
            r = np.linalg.norm(bx[i] - ax[i] / ref_m["ew"][a, i])
            assert abs(r - ref_m["res"][a, i]) <= 1e-3 * ref_m["res"][a, i] + 1e-14
    # per-instance counts: the sweep adds at least 2k FP64 applies per instance
    assert np.all(ref_m["stats"][:, 2] >= raw["stats"][:, 2] + 2 * k)
    plan.close()


@pytest.mark.parametrize("refine_tol", [1e-9, 1e-12])
def test_refinement_with_tight_search_solve(cuda, fame_lib, refine_tol):
    """The sweep's search directions W = B^-1 R solved far below the size of
    the residuals R (~1e-10 and less): every complex64 round of the mixed
    solve sees a right-hand side scaled to norm [1, 2), so no CG product
    underflows and the band solve completes with residuals no larger than
    before the sweep."""
    n, k = 12, 6
    plan = fame.woodpile_plan(n, [fame.fcc_point("X"), fame.fcc_point("L")])
    plan.set_option("refine_tol", refine_tol)
    m = plan.band_solve(k, tol=1e-8, prec="c64", inner_tol=3e-12, p=2 * k + 4)
    assert m["status"] == 0
    assert np.all(m["res"] <= m["res_before"])
    assert m["res"].max() <= 1e-8
    plan.close()


def test_relaxed_inner_tolerance(cuda, fame_lib):
    """FAME_OPT_RELAX: the inner solves of the late Lanczos vectors may be
    looser once the wanted Ritz residuals are small.  Against no relaxation:
    about the same Lanczos steps, eigenvalues of the FP64 form to 1e-9, NFSEP
    residuals below the bar, and no more inner CG iterations."""
    n, k = 12, 6
    kv = [fame.fcc_point("X"), fame.fcc_point("L")]
    plan = fame.woodpile_plan(n, kv)
    ref = plan.band_solve(k, tol=1e-11, prec="c128", inner_tol=1e-13, p=2 * k)
    out = {}
    for c in (0.0, 0.1, 0.5):
        plan.set_option("relax", c)
        out[c] = plan.band_solve(k, tol=1e-8, prec="c64", inner_tol=3e-12, p=2 * k + 4)
        assert out[c]["status"] == 0
        assert out[c]["res"].max() <= 1e-8
        assert np.allclose(out[c]["ew"], ref["ew"], rtol=1e-9, atol=0)
    steps0 = out[0.0]["stats"][:, 0].sum()
    for c in (0.1, 0.5):
        assert abs(out[c]["stats"][:, 0].sum() - steps0) <= 0.1 * steps0
    assert out[0.5]["stats"][:, 3].sum() <= out[0.0]["stats"][:, 3].sum()
    with pytest.raises(fame.FameError):
        plan.set_option("relax", 1.5)
    plan.close()
