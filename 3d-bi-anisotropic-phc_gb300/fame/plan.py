"""Python view of a FAME plan: one cubic n^3 grid, ``nk`` k-point instances.

Vectors are torch tensors on the CUDA device (complex128 -> the FP64 path,
complex64 -> the complex64 path) of shape (nvec, L) or (L,), or NumPy arrays
on the host (staged by the library).  Calls run on torch's current CUDA
stream.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check, load
from .setup import covariant_blocks

try:
    import torch
except ImportError:  # pragma: no cover - torch is required on the GPU path
    torch = None


def _prec_of(x):
    if torch is not None and isinstance(x, torch.Tensor):
        if x.dtype == torch.complex128:
            return L.FAME_C128
        if x.dtype == torch.complex64:
            return L.FAME_C64
        raise TypeError(f"unsupported dtype {x.dtype}")
    x = np.asarray(x)
    if x.dtype == np.complex128:
        return L.FAME_C128
    if x.dtype == np.complex64:
        return L.FAME_C64
    raise TypeError(f"unsupported dtype {x.dtype}")


def _tune_prec(prec):
    """Tuning key of 'c64', 'c128' or 'c128ds' (complex128 vectors, double-single
    arithmetic: the mixed inner solves' residuals), or the FAME_* code itself."""
    if prec in ("c64", L.FAME_C64):
        return L.FAME_C64
    if prec in ("c128ds", L.FAME_C128_DS):
        return L.FAME_C128_DS
    return L.FAME_C128


class Plan:
    """``fame_plan_create`` wrapper (replaces the per-k mtx_A / mtx_B / fnc setup)."""

    def __init__(self, n: int, thetas, phase, tensors):
        self._lib = load()
        self.n = int(n)
        th = np.ascontiguousarray(np.asarray(thetas, dtype=np.float64).reshape(-1, 3))
        self.nk = th.shape[0]
        self.thetas = th
        ph = np.ascontiguousarray(np.asarray(phase, dtype=np.uint8).reshape(-1))
        if ph.size != self.n ** 3:
            raise ValueError("phase must hold n^3 vertex ids")
        t = np.asarray(tensors, dtype=np.complex128)
        if t.ndim == 2:
            t = np.broadcast_to(t, (self.nk,) + t.shape)
        t = np.ascontiguousarray(t.reshape(self.nk, -1, 27))
        self.nphase = t.shape[1]
        self.tensors = t
        self.phase = ph
        self._h = C.c_void_p()
        pd = C.POINTER(C.c_double)
        rc = self._lib.fame_plan_create(C.byref(self._h), self.n, self.nk, th.ctypes.data_as(pd),
                                        ph.ctypes.data_as(C.POINTER(C.c_uint8)), self.nphase,
                                        t.view(np.float64).ctypes.data_as(pd))
        check(rc, None, "fame_plan_create")
        self.Nq = self.n ** 3

    @classmethod
    def from_phases(cls, n, thetas, phase, constitutive_per_phase, A=None):
        """Plan from per-phase 6x6 constitutive blocks (shared by all instances,
        or one list per instance)."""
        c = np.asarray(constitutive_per_phase, dtype=np.complex128)
        if c.ndim == 3:
            tens = np.stack([covariant_blocks(m, A) for m in c])
        else:
            tens = np.stack([np.stack([covariant_blocks(m, A) for m in ci]) for ci in c])
        return cls(n, thetas, phase, tens)

    @classmethod
    def from_fields(cls, n, thetas, eps, gamma, lattice=None):
        """Field-mode plan (fame_plan_create_field): per-vertex eps(r) I, mu = I,
        xi = -zeta = i gamma(r) I on the n^3 vertices (x fastest)."""
        from .setup import fcc_lattice
        self = cls.__new__(cls)
        self._lib = load()
        self.n = int(n)
        th = np.ascontiguousarray(np.asarray(thetas, dtype=np.float64).reshape(-1, 3))
        self.nk = th.shape[0]
        self.thetas = th
        A = fcc_lattice() if lattice is None else np.asarray(lattice, dtype=np.float64)
        self.lattice = np.ascontiguousarray(A.reshape(3, 3))
        self.Nq = self.n ** 3
        self.nphase = 1
        self.phase = None
        self.tensors = None
        e, g = self._field_arrays(eps, gamma)
        self._h = C.c_void_p()
        pd = C.POINTER(C.c_double)
        rc = self._lib.fame_plan_create_field(C.byref(self._h), self.n, self.nk, th.ctypes.data_as(pd),
                                              self.lattice.ctypes.data_as(pd), e.ctypes.data_as(pd),
                                              g.ctypes.data_as(pd))
        check(rc, None, "fame_plan_create_field")
        return self

    def _field_arrays(self, eps, gamma):
        def host(a):
            if torch is not None and isinstance(a, torch.Tensor):
                a = a.detach().cpu().numpy()
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
            if a.size != self.Nq:
                raise ValueError("fields must hold n^3 vertex values")
            return a
        return host(eps), host(gamma)

    def set_fields(self, eps, gamma):
        """fame_set_field: replace the per-vertex fields of a field-mode plan."""
        e, g = self._field_arrays(eps, gamma)
        pd = C.POINTER(C.c_double)
        check(self._lib.fame_set_field(self._h, e.ctypes.data_as(pd), g.ctypes.data_as(pd)), self._h,
              "fame_set_field")
        return self

    def eig_gradient(self, ev, omega, weight=None, inst=None, out=None, accumulate=False):
        """fame_eig_gradient: sum_v weight_v d omega_v / d(eps, gamma) at every
        vertex.  ev: complex128 CUDA tensor (nvec, 4Nq); omega, weight (nvec,).
        Returns (g_eps, g_gamma, xBx): FP64 CUDA tensors (Nq,) and a NumPy array."""
        ev = ev.reshape(-1, 4 * self.Nq).contiguous()
        if ev.dtype != torch.complex128:
            raise TypeError("eigenvectors must be complex128")
        nvec = ev.shape[0]
        om = np.ascontiguousarray(np.broadcast_to(np.asarray(omega, dtype=np.float64), (nvec,)))
        wt = np.ones(nvec) if weight is None else np.asarray(weight, dtype=np.float64)
        wt = np.ascontiguousarray(np.broadcast_to(wt, (nvec,)))
        if out is None:
            g_e = torch.zeros(self.Nq, dtype=torch.float64, device=ev.device)
            g_g = torch.zeros(self.Nq, dtype=torch.float64, device=ev.device)
        else:
            g_e, g_g = out
        ip = None
        if inst is not None:
            ia = np.ascontiguousarray(np.broadcast_to(np.asarray(inst, dtype=np.int32), (nvec,)))
            ip = ia.ctypes.data_as(C.POINTER(C.c_int))
        xbx = np.zeros(nvec)
        pd = C.POINTER(C.c_double)
        self._stream()
        rc = self._lib.fame_eig_gradient(self._h, nvec, ip, C.c_void_p(ev.data_ptr()), om.ctypes.data_as(pd),
                                         wt.ctypes.data_as(pd), C.c_void_p(g_e.data_ptr()),
                                         C.c_void_p(g_g.data_ptr()), int(bool(accumulate)), xbx.ctypes.data_as(pd))
        check(rc, self._h, "fame_eig_gradient")
        return g_e, g_g, xbx

    def restore(self, ev, omega, inst=None, want_fields=True, outside_only=False):
        """fame_restore: E, H fields (Eigen_Restoration_Chiral_no_inv.m), the
        ORGSEP residual (EvaluteError_Chiral_no_inv.m:19) and max |e_c|, |h_c|
        (Fig6cd_plot_max_field.m).  Returns dict(E, H, res_orgsep, max_e, max_h)."""
        ev = ev.reshape(-1, 4 * self.Nq).contiguous()
        if ev.dtype != torch.complex128:
            raise TypeError("eigenvectors must be complex128")
        nvec = ev.shape[0]
        om = np.ascontiguousarray(np.broadcast_to(np.asarray(omega, dtype=np.float64), (nvec,)))
        E = H = None
        if want_fields:
            E = torch.empty((nvec, 3 * self.Nq), dtype=torch.complex128, device=ev.device)
            H = torch.empty_like(E)
        res = np.zeros(nvec)
        me = np.zeros(nvec)
        mh = np.zeros(nvec)
        ip = None
        if inst is not None:
            ia = np.ascontiguousarray(np.broadcast_to(np.asarray(inst, dtype=np.int32), (nvec,)))
            ip = ia.ctypes.data_as(C.POINTER(C.c_int))
        pd = C.POINTER(C.c_double)
        self._stream()
        rc = self._lib.fame_restore(self._h, nvec, ip, C.c_void_p(ev.data_ptr()), om.ctypes.data_as(pd),
                                    C.c_void_p(E.data_ptr()) if E is not None else None,
                                    C.c_void_p(H.data_ptr()) if H is not None else None, res.ctypes.data_as(pd),
                                    me.ctypes.data_as(pd), mh.ctypes.data_as(pd), int(bool(outside_only)))
        check(rc, self._h, "fame_restore")
        return dict(E=E, H=H, res_orgsep=res, max_e=me, max_h=mh)

    # -- life cycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.fame_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def raw(self):
        """The fame_plan_t handle (ctypes c_void_p) for direct C-ABI calls."""
        return self._h

    def _stream(self):
        if torch is not None and torch.cuda.is_available():
            self._lib.fame_set_stream(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream))

    def sync(self):
        check(self._lib.fame_sync(self._h), self._h, "fame_sync")

    def set_option(self, option, value):
        """fame_set_option: 'precond' (bool), 'tol32' (float), 'graph' (0, 1 or 2), 'itol_floor' (float),
        'plane_split' (bool), 'sira_nearest' (bool), 'refine' (bool), 'refine_tol' (float),
        'pi_table' (bool), 'c64_round' (bool), 'relax' (float in [0, 1)), 'relax_max' (float >= 1) or
        'ds_residual' (bool)."""
        code = {"precond": L.FAME_OPT_PRECOND, "tol32": L.FAME_OPT_TOL32, "graph": L.FAME_OPT_GRAPH,
                "itol_floor": L.FAME_OPT_ITOL_FLOOR, "plane_split": L.FAME_OPT_PLANE_SPLIT,
                "sira_nearest": L.FAME_OPT_SIRA_NEAREST, "refine": L.FAME_OPT_REFINE,
                "refine_tol": L.FAME_OPT_REFINE_TOL, "pi_table": L.FAME_OPT_PI_TABLE,
                "c64_round": L.FAME_OPT_C64_ROUND, "relax": L.FAME_OPT_RELAX,
                "relax_max": L.FAME_OPT_RELAX_MAX, "ds_residual": L.FAME_OPT_DS_RESIDUAL}.get(option, option)
        check(self._lib.fame_set_option(self._h, int(code), float(value)), self._h, "fame_set_option")
        return self

    def autotune(self, nvec=None, prec="c64", cache=None):
        """fame_autotune for batch width `nvec` (default: the plan's instance
        count).  With `cache` (a JSON file path) a setting measured before on
        the same device, grid, precision and width is installed without
        re-timing, and new measurements are added to the file.
        Returns dict(chunk, stencil_tpb, lanes, us, cached) (lanes: threads
        per FFT pencil of the plane kernels, -1 the size's default)."""
        import json
        import os
        nvec = self.nk if nvec is None else int(nvec)
        pr = _tune_prec(prec)
        dev = torch.cuda.get_device_name() if torch is not None and torch.cuda.is_available() else "gpu"
        key = f"{dev}|n={self.n}|{ {L.FAME_C64: 'c64', L.FAME_C128: 'c128'}.get(pr, 'c128ds') }|nvec={nvec}"
        table = {}
        if cache and os.path.exists(cache):
            with open(cache) as f:
                table = json.load(f)
        if key in table:
            t = table[key]
            self.set_tune(pr, nvec, t["chunk"], t["stencil_tpb"], t.get("lanes", -1))
            return dict(t, cached=True)
        ch, tpb, us, ln = C.c_int(), C.c_int(), C.c_double(), C.c_int()
        self._stream()
        check(self._lib.fame_autotune(self._h, pr, nvec, C.byref(ch), C.byref(tpb), C.byref(us)), self._h,
              "fame_autotune")
        check(self._lib.fame_get_tune(self._h, pr, nvec, None, None, C.byref(ln)), self._h, "fame_get_tune")
        t = dict(chunk=ch.value, stencil_tpb=tpb.value, lanes=ln.value, us=us.value)
        if cache:
            table[key] = t
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return dict(t, cached=False)

    def autotune_mixed(self, nvec=None, cache=None):
        """The launch parameters the mixed form uses: complex64 fncB (inner CG)
        and, where the grid has it, the double-single fncB (the inner solves'
        residuals).  Returns {'c64': ..., 'c128ds': ... or None}."""
        out = {"c64": self.autotune(nvec=nvec, prec="c64", cache=cache), "c128ds": None}
        try:
            out["c128ds"] = self.autotune(nvec=nvec, prec="c128ds", cache=cache)
        except L.FameError as e:
            if e.code != L.FAME_ERR_UNSUPPORTED:
                raise
        return out

    def set_tune_mixed(self, nvec, tunes):
        """Installs what autotune_mixed returned (on another plan of the same
        grid and batch width)."""
        for prec, t in tunes.items():
            if t:
                self.set_tune(prec, nvec, t["chunk"], t["stencil_tpb"], t.get("lanes", -1))

    def set_tune(self, prec, nvec, chunk, stencil_tpb, lanes=-1):
        """fame_set_tune + fame_set_tune_lanes: install fncB launch parameters
        measured before (on another plan of the same grid, precision and
        batch width)."""
        pr = _tune_prec(prec)
        check(self._lib.fame_set_tune(self._h, pr, int(nvec), int(chunk), int(stencil_tpb)), self._h,
              "fame_set_tune")
        check(self._lib.fame_set_tune_lanes(self._h, pr, int(nvec), int(lanes)), self._h, "fame_set_tune_lanes")

    def get_tune(self, prec, nvec):
        """fame_get_tune: the installed dict(chunk, stencil_tpb, lanes)."""
        pr = _tune_prec(prec)
        ch, tpb, ln = C.c_int(), C.c_int(), C.c_int()
        check(self._lib.fame_get_tune(self._h, pr, int(nvec), C.byref(ch), C.byref(tpb), C.byref(ln)), self._h,
              "fame_get_tune")
        return dict(chunk=ch.value, stencil_tpb=tpb.value, lanes=ln.value)

    # -- generic call -------------------------------------------------------
    def _call(self, fn, x, out_len, inst, *extra, name=""):
        prec = _prec_of(x)
        is_torch = torch is not None and isinstance(x, torch.Tensor)
        single = x.ndim == 1
        if is_torch:
            xx = x.reshape(1, -1) if single else x
            xx = xx.contiguous()
            nvec = xx.shape[0]
            y = torch.empty((nvec, out_len), dtype=xx.dtype, device=xx.device)
            xp, yp, flags = C.c_void_p(xx.data_ptr()), C.c_void_p(y.data_ptr()), 0
            self._stream()
        else:
            xx = np.ascontiguousarray(np.asarray(x).reshape(1, -1) if single else np.asarray(x))
            nvec = xx.shape[0]
            y = np.empty((nvec, out_len), dtype=xx.dtype)
            xp, yp, flags = C.c_void_p(xx.ctypes.data), C.c_void_p(y.ctypes.data), L.FAME_HOST_PTR
        ip = None
        if inst is not None:
            ia = np.ascontiguousarray(np.broadcast_to(np.asarray(inst, dtype=np.int32), (nvec,)))
            ip = ia.ctypes.data_as(C.POINTER(C.c_int))
        rc = fn(self._h, prec, *extra[:1], xp, yp, nvec, ip, *extra[1:], flags) if extra else \
            fn(self._h, prec, xp, yp, nvec, ip, flags)
        check(rc, self._h, name)
        return y.reshape(-1) if single else y

    # -- operator handles ---------------------------------------------------
    def apply_A(self, x, inst=None):
        """fncA (fun_Lanczos/fncA.m)."""
        return self._call(self._lib.fame_apply_A, x, 4 * self.Nq, inst, name="fame_apply_A")

    def apply_B(self, x, inst=None):
        """fncB (fun_Lanczos/fncB.m)."""
        return self._call(self._lib.fame_apply_B, x, 4 * self.Nq, inst, name="fame_apply_B")

    def transform(self, x, trans: int, inst=None):
        """MtxVecMul_FFT: trans 0 'notranspose', 1 'transpose' (3Nq vectors)."""
        return self._call(self._lib.fame_curl_transform, x, 3 * self.Nq, inst, int(trans), name="fame_curl_transform")

    def handle(self, which: int, x, inst=None):
        """fnc.Pr / Qr / Prs / Qrs (Funhand_Generate_Lanzcos.m:79-82)."""
        out = 3 * self.Nq if which in (L.FAME_PR, L.FAME_QR) else 2 * self.Nq
        return self._call(self._lib.fame_apply_handle, x, out, inst, int(which), name="fame_apply_handle")

    def material(self, x, inst=None):
        """[M_int J_int'; J_int N_int] on 6Nq Bloch-frame vectors."""
        return self._call(self._lib.fame_apply_material, x, 6 * self.Nq, inst, name="fame_apply_material")

    def apply_Binv(self, x, tol=1e-12, maxit=10000, inst=None, raise_on_noconv=False):
        """fncinvB: CG on B (fun_Lanczos/fncinvB.m).  Returns (y, iters, relres)."""
        prec = _prec_of(x)
        is_torch = torch is not None and isinstance(x, torch.Tensor)
        single = x.ndim == 1
        if is_torch:
            xx = (x.reshape(1, -1) if single else x).contiguous()
            nvec = xx.shape[0]
            y = torch.empty_like(xx)
            xp, yp, flags = C.c_void_p(xx.data_ptr()), C.c_void_p(y.data_ptr()), 0
            self._stream()
        else:
            xx = np.ascontiguousarray(np.asarray(x).reshape(1, -1) if single else np.asarray(x))
            nvec = xx.shape[0]
            y = np.empty_like(xx)
            xp, yp, flags = C.c_void_p(xx.ctypes.data), C.c_void_p(y.ctypes.data), L.FAME_HOST_PTR
        its = np.zeros(nvec, dtype=np.int32)
        rr = np.zeros(nvec, dtype=np.float64)
        ip = None
        if inst is not None:
            ia = np.ascontiguousarray(np.broadcast_to(np.asarray(inst, dtype=np.int32), (nvec,)))
            ip = ia.ctypes.data_as(C.POINTER(C.c_int))
        rc = self._lib.fame_apply_Binv(self._h, prec, xp, yp, nvec, ip, float(tol), int(maxit),
                                       its.ctypes.data_as(C.POINTER(C.c_int)),
                                       rr.ctypes.data_as(C.POINTER(C.c_double)), flags)
        if rc != L.FAME_OK and (rc != L.FAME_ERR_NOT_CONVERGED or raise_on_noconv):
            check(rc, self._h, "fame_apply_Binv")
        return (y.reshape(-1) if single else y), its, rr

    # -- solvers ------------------------------------------------------------
    def lanczos(self, k, tol=1e-10, maxit=10000, p=None, v0=None, inst=0, prec="c128", inner_tol=1e-12,
                want_vectors=True):
        """Thick-restart Lanczos (fun_Lanczos/Lanczos.m) on instance `inst`.

        Returns dict(ew, omega, res, ev, stats, status)."""
        p = 2 * k if p is None else p
        ew = np.zeros(k, dtype=np.float64)
        res = np.zeros(k, dtype=np.float64)
        stats = np.zeros(4, dtype=np.int64)
        pd = C.POINTER(C.c_double)
        v0p = None
        if v0 is not None:
            v0a = np.ascontiguousarray(np.asarray(v0, dtype=np.complex128).reshape(-1))
            v0p = v0a.view(np.float64).ctypes.data_as(pd)
        ev = None
        evp = None
        if want_vectors:
            ev = torch.empty((k, 4 * self.Nq), dtype=torch.complex128, device="cuda")
            evp = C.c_void_p(ev.data_ptr())
        self._stream()
        pr = L.FAME_C64 if prec in ("c64", "mixed", L.FAME_C64) else L.FAME_C128
        rc = self._lib.fame_lanczos(self._h, pr, int(inst), int(k), float(tol), int(maxit), int(p), v0p,
                                    float(inner_tol), ew.ctypes.data_as(pd), evp, res.ctypes.data_as(pd),
                                    stats.ctypes.data_as(C.POINTER(C.c_longlong)))
        if rc not in (L.FAME_OK, L.FAME_ERR_NOT_CONVERGED):
            check(rc, self._h, "fame_lanczos")
        return dict(ew=ew, omega=1.0 / ew, res=res, ev=ev, stats=stats, status=rc,
                    res_before=self.refine_residuals(res.shape))

    def jdsira(self, nev, target=0.0, tol=1e-8, no_restart=50, restart_dim=4, inner_tol=1e-2, inner_maxit=30000,
               inst=0, inner_prec="c64", want_vectors=False, shift=0.0):
        """SIRA with locking (GEP_AB_Herm_JDSIRA_Driver4.m called as Driver4(fncB, fncA, ...)):
        the `nev` eigenvalues of fncB x = theta fncA x closest to `target`.
        Returns dict(ew, res, ev, stats, status)."""
        ew = np.zeros(nev, dtype=np.float64)
        res = np.zeros(nev, dtype=np.float64)
        stats = np.zeros(4, dtype=np.int64)
        pd = C.POINTER(C.c_double)
        ev = None
        evp = None
        if want_vectors:
            ev = torch.empty((nev, 4 * self.Nq), dtype=torch.complex128, device="cuda")
            evp = C.c_void_p(ev.data_ptr())
        self._stream()
        pr = L.FAME_C64 if inner_prec in ("c64", L.FAME_C64) else L.FAME_C128
        rc = self._lib.fame_jdsira(self._h, pr, int(inst), int(nev), float(target), float(shift), float(tol),
                                   int(no_restart),
                                   int(restart_dim), float(inner_tol), int(inner_maxit), ew.ctypes.data_as(pd), evp,
                                   res.ctypes.data_as(pd), stats.ctypes.data_as(C.POINTER(C.c_longlong)))
        if rc not in (L.FAME_OK, L.FAME_ERR_NOT_CONVERGED):
            check(rc, self._h, "fame_jdsira")
        return dict(ew=ew, res=res, ev=ev, stats=stats, status=rc)

    def band_solve(self, k, tol=1e-10, maxit=10000, p=None, prec="c64", inner_tol=1e-12, want_vectors=False):
        """All instances at once (fame_band_solve).  Returns dict(ew, omega, res,
        stats, status, ev) with ev a complex128 CUDA tensor (nk, k, 4Nq) or None."""
        p = 2 * k if p is None else p
        ew = np.zeros((self.nk, k), dtype=np.float64)
        res = np.zeros((self.nk, k), dtype=np.float64)
        stats = np.zeros((self.nk, 4), dtype=np.int64)
        pd = C.POINTER(C.c_double)
        ev = None
        evp = None
        if want_vectors:
            ev = torch.empty((self.nk, k, 4 * self.Nq), dtype=torch.complex128, device="cuda")
            evp = C.c_void_p(ev.data_ptr())
        self._stream()
        pr = L.FAME_C64 if prec in ("c64", "mixed", L.FAME_C64) else L.FAME_C128
        rc = self._lib.fame_band_solve(self._h, pr, int(k), float(tol), int(maxit), int(p), float(inner_tol),
                                       ew.ctypes.data_as(pd), evp, res.ctypes.data_as(pd),
                                       stats.ctypes.data_as(C.POINTER(C.c_longlong)))
        if rc not in (L.FAME_OK, L.FAME_ERR_NOT_CONVERGED):
            check(rc, self._h, "fame_band_solve")
        return dict(ew=ew, omega=1.0 / ew, res=res, stats=stats, status=rc, ev=ev,
                    res_before=self.refine_residuals(res.shape))

    def refine_residuals(self, shape=None):
        """NFSEP residuals before the last FP64 refinement sweep (fame_refine_residuals), or None."""
        n = self._lib.fame_refine_residuals(self._h, None, 0)
        if n <= 0:
            return None
        out = np.zeros(n, dtype=np.float64)
        self._lib.fame_refine_residuals(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), n)
        return out.reshape(shape) if shape is not None and int(np.prod(shape)) == n else out
