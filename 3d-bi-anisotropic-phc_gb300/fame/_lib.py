"""ctypes binding of the FAME GB300 C ABI (``include/fame.h``).

The shared library is built in-tree by ``fame.build.build_library()`` (called
by ``__graft_entry__.build()``).  There is no fallback: if the library is
missing, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBNAME = "libfame_gb300.so"

FAME_OK = 0
FAME_ERR_BAD_ARG = 1
FAME_ERR_CUDA = 2
FAME_ERR_NOT_CONVERGED = 3
FAME_ERR_BREAKDOWN = 4
FAME_ERR_NAN = 5
FAME_ERR_UNSUPPORTED = 6
FAME_ERR_SINGULAR = 7
FAME_ERR_ALLOC = 8
FAME_C128 = 0
FAME_C64 = 1
FAME_C128_DS = 2
FAME_PR, FAME_QR, FAME_PRS, FAME_QRS = 0, 1, 2, 3
FAME_HOST_PTR = 1
FAME_OPT_PRECOND = 0
FAME_OPT_TOL32 = 1
FAME_OPT_GRAPH = 2
FAME_OPT_ITOL_FLOOR = 3
FAME_OPT_PLANE_SPLIT = 4
FAME_OPT_SIRA_NEAREST = 5
FAME_OPT_REFINE = 6
FAME_OPT_REFINE_TOL = 7
FAME_OPT_PI_TABLE = 8
FAME_OPT_C64_ROUND = 9
FAME_OPT_RELAX = 10
FAME_OPT_RELAX_MAX = 11
FAME_OPT_DS_RESIDUAL = 12
FAME_SHAPE_WOODPILE, FAME_SHAPE_SPHERE, FAME_SHAPE_TETRA = 0, 1, 2
FAME_RASTER_PAINT = 2

STATUS_NAMES = {0: "OK", 1: "BAD_ARG", 2: "CUDA", 3: "NOT_CONVERGED", 4: "BREAKDOWN", 5: "NAN",
                6: "UNSUPPORTED", 7: "SINGULAR", 8: "ALLOC"}

_lib = None

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_pi = C.POINTER(C.c_int)
_pd = C.POINTER(C.c_double)
_pll = C.POINTER(C.c_longlong)

SIGNATURES = {
    "fame_version": (C.c_char_p, []),
    "fame_kernel_launches": (C.c_longlong, []),
    "fame_host_launches": (C.c_longlong, []),
    "fame_plan_create": (_i, [C.POINTER(_vp), _i, _i, _pd, C.POINTER(C.c_uint8), _i, _pd]),
    "fame_plan_destroy": (_i, [_vp]),
    "fame_set_stream": (_i, [_vp, _vp]),
    "fame_set_option": (_i, [_vp, _i, _d]),
    "fame_sync": (_i, [_vp]),
    "fame_last_error": (C.c_char_p, [_vp]),
    "fame_refine_residuals": (C.c_int, [_vp, C.POINTER(C.c_double), C.c_int]),
    "fame_plan_info": (_i, [_vp, _pi, _pi, _pll]),
    "fame_apply_A": (_i, [_vp, _i, _vp, _vp, _i, _pi, _i]),
    "fame_apply_B": (_i, [_vp, _i, _vp, _vp, _i, _pi, _i]),
    "fame_apply_B_noalloc": (_i, [_vp, _i, _vp, _vp, _i]),
    "fame_apply_Binv": (_i, [_vp, _i, _vp, _vp, _i, _pi, _d, _i, _pi, _pd, _i]),
    "fame_curl_transform": (_i, [_vp, _i, _i, _vp, _vp, _i, _pi, _i]),
    "fame_apply_handle": (_i, [_vp, _i, _i, _vp, _vp, _i, _pi, _i]),
    "fame_apply_material": (_i, [_vp, _i, _vp, _vp, _i, _pi, _i]),
    "fame_lanczos": (_i, [_vp, _i, _i, _i, _d, _i, _i, _pd, _d, _pd, _vp, _pd, _pll]),
    "fame_band_solve": (_i, [_vp, _i, _i, _d, _i, _i, _d, _pd, _vp, _pd, _pll]),
    "fame_material_blocks": (_i, [_pd, _pd, _pd]),
    "fame_jdsira": (_i, [_vp, _i, _i, _i, _d, _d, _d, _i, _i, _d, _i, _pd, _vp, _pd, _pll]),
    "fame_plan_create_field": (_i, [C.POINTER(_vp), _i, _i, _pd, _pd, _pd, _pd]),
    "fame_set_field": (_i, [_vp, _pd, _pd]),
    "fame_eig_gradient": (_i, [_vp, _i, _pi, _vp, _pd, _pd, _vp, _vp, _i, _pd]),
    "fame_restore": (_i, [_vp, _i, _pi, _vp, _pd, _vp, _vp, _pd, _pd, _pd, _i]),
    "fame_autotune": (_i, [_vp, _i, _i, _pi, _pi, _pd]),
    "fame_set_tune": (_i, [_vp, _i, _i, _i, _i]),
    "fame_set_tune_lanes": (_i, [_vp, _i, _i, _i]),
    "fame_get_tune": (_i, [_vp, _i, _i, _pi, _pi, _pi]),
    "fame_rasterize": (_i, [_i, _pd, _i, _pd, _i, _vp, _i]),
}


class FameError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"FAME {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib_path() -> str:
    return os.path.join(HERE, LIBNAME)


def load():
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        p = lib_path()
        if not os.path.exists(p):
            raise RuntimeError(f"FAME CUDA library not built ({p}); run __graft_entry__.build()")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(code: int, plan_handle=None, what: str = ""):
    if code != FAME_OK:
        msg = load().fame_last_error(plan_handle)
        raise FameError(code, (what + ": " if what else "") + (msg.decode() if msg else ""))
    return code
