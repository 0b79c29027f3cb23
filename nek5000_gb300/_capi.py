"""ctypes binding of libnekgpu.so (the C ABI declared in include/nekgpu.h).

The library is the product: this module only loads it and declares the
argument types.  If the shared object is missing the import fails loudly --
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnekgpu.so")

OK = 0
EINVAL, EHANDLE, ECUDA, ENOMEM, ENOTCONV, ENOSETUP, ENAN, EIO = -1, -2, -3, -4, -5, -6, -7, -8
OPT_EXACT, OPT_TIMING, OPT_CHUNK, OPT_ISTEP, OPT_TMA, OPT_GRAPH, OPT_MIXED_MODE = (
    1, 2, 3, 4, 5, 6, 7)
OPT_AUTOTUNE = 8
OPT_SPLIT = 9
OPT_DF = 10
OPT_FACE_ORDER = 11
OPT_COARSE = 12
MAX_LX1 = 12
NOALLOC_MAX_POINTS = 4194304
PROJ_SPACES, PROJ_MAX, PROJ_DEFAULT = 16, 16, 8
MULTI_MAX = 3
GMRES_MAX = 50

STATUS_NAMES = {
    0: "NEKGPU_OK", -1: "NEKGPU_EINVAL", -2: "NEKGPU_EHANDLE", -3: "NEKGPU_ECUDA",
    -4: "NEKGPU_ENOMEM", -5: "NEKGPU_ENOTCONV", -6: "NEKGPU_ENOSETUP", -7: "NEKGPU_ENAN",
    -8: "NEKGPU_EIO",
}

# Every exported entry point and its argument types.  Pointer arguments are
# passed as c_void_p so that host buffers (numpy) and device buffers (torch
# data_ptr) go through the same declaration.
_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    # mesh ingestion (include/nekmesh.h): host code
    "nekmesh_last_error": [C.c_char_p, _IP],
    "nekmesh_re2_open": [C.c_char_p, _I64P],
    "nekmesh_re2_header": [_I64P, _IP, _IP, _IP, _IP, _I64P, _IP],
    "nekmesh_re2_xyz": [_I64P, _P, _P, _P, _P],
    "nekmesh_re2_curves": [_I64P, _P, _P, _P, _P],
    "nekmesh_re2_bc": [_I64P, _IP, _P, _P],
    "nekmesh_re2_close": [_I64P],
    "nekmesh_co2_read": [C.c_char_p, _IP, _IP, _IP, _P],
    "nekmesh_co2_write": [C.c_char_p, _IP, _IP, _IP, _P],
    "nekmesh_ma2_read": [C.c_char_p, _IP, _IP, _P, _P],
    "nekmesh_amg_setup": [_I64P, _P, _P, _P, _I64P],
    "nekmesh_amg_layout": [_I64P, _IP, _P, _P],
    "nekmesh_amg_level": [_I64P, _IP, _P, _IP, _DP] + [_P] * 13,
    "nekmesh_amg_apply": [_I64P, _P, _P],
    "nekmesh_amg_free": [_I64P],
    "nekmesh_connect": [_IP, _IP, _P, _P, _P, _P, _P, _DP, _P, _I64P],
    "nekmesh_setvert3d": [_IP, _IP, _P, _P, _I64P],
    "nekmesh_check_p_bc": [_IP, _IP, C.c_char_p, _P],
    "nekmesh_xyzlin": [_IP, _IP, _P, _P, _P, _P, _P, _P, _P],
    "nekmesh_genxyz": [_IP, _IP, _P, _P, _P, _P, _I64P, _P, _P, _P, C.c_char_p, _P, _P, _P],
    # solve path (include/nekgpu.h)
    "nekgpu_init": [_IP, _I64P],
    "nekgpu_finalize": [_I64P],
    "nekgpu_last_error": [_I64P, C.c_char_p, _IP],
    "nekgpu_set_option": [_I64P, _IP, _IP],
    "nekgpu_setup": [_I64P, _IP, _IP, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "nekgpu_hmh_gmres_dev": [_I64P, _P, _P, _P, _P, _P, _DP, _IP, _IP, _IP, _IP, _DP, _DP],
    "nekgpu_hmh_gmres": [_I64P, _P, _P, _P, _P, _P, _DP, _IP, _IP, _IP, _IP, _DP, _DP],
    "nekgpu_hmh_flex_cg_dev": [_I64P, _P, _P, _P, _P, _P, _DP, _IP, _IP, _IP, _DP, _DP],
    "nekgpu_hmh_flex_cg": [_I64P, _P, _P, _P, _P, _P, _DP, _IP, _IP, _IP, _DP, _DP],
    "nekgpu_wgradm1_dev": [_I64P, _P, _P, _P, _P],
    "nekgpu_dudxyz_dev": [_I64P, _P, _P, _IP],
    "nekgpu_cdtp_dev": [_I64P, _P, _P, _IP],
    "nekgpu_op_curl_dev": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _P],
    "nekgpu_dealias_setup": [_I64P, _IP],
    "nekgpu_convop_dev": [_I64P] + [_P] * 5,
    "nekgpu_convect_cons_dev": [_I64P] + [_P] * 5,
    "nekgpu_conv2_dev": [_I64P] + [_P] * 5,
    "nekgpu_convopo_dev": [_I64P] + [_P] * 6,
    "nekgpu_conv1_dev": [_I64P] + [_P] * 5,
    "nekgpu_advab_dev": [_I64P] + [_P] * 6,
    "nekgpu_makeabf_dev": [_I64P, _P, _P, _P, _P, _P],
    "nekgpu_makebdf_dev": [_I64P, _P, _P, _P, _P, _P, _IP, _DP],
    "nekgpu_sumab_dev": [_I64P, _P, _P, _P, _P, _IP],
    "nekgpu_cresvsp_dev": [_I64P] + [_P] * 14,
    "nekgpu_cresvsp_weak_dev": [_I64P] + [_P] * 14 + [_IP],
    "nekgpu_axhmsf_dev": [_I64P] + [_P] * 8,
    "nekgpu_hmhzsf_dev": [_I64P] + [_P] * 13 + [_DP, _IP, _DP, _DP],
    "nekgpu_crespsp_dev": [_I64P] + [_P] * 12 + [_DP, _IP, _P, _P, _P, _P],
    "nekgpu_col2_dev": [_I64P, _P, _P],
    "nekgpu_col3_dev": [_I64P, _P, _P, _P],
    "nekgpu_add2s1_dev": [_I64P, _P, _P, _DP],
    "nekgpu_add2s2_dev": [_I64P, _P, _P, _DP],
    "nekgpu_vlsc3_dev": [_I64P, _P, _P, _P, _DP],
    "nekgpu_vlsc32_dev": [_I64P, _P, _P, _P, _DP],
    "nekgpu_invcol1_dev": [_I64P, _P],
    "nekgpu_vlmax_dev": [_I64P, _P, _IP, _DP],
    "nekgpu_setprec_local_dev": [_I64P, _P, _P, _P],
    "nekgpu_iface_setup": [_I64P, _I64P, _P, _P],
    "nekgpu_iface_gather_dev": [_I64P, _P, _P],
    "nekgpu_iface_scatter_dev": [_I64P, _P, _P],
    "nekgpu_h1mg_setup": [_I64P, _P, _P, _P, _P, _P, _P, _IP],
    "nekgpu_h1mg_free": [_I64P],
    "nekgpu_h1mg_apply_dev": [_I64P, _P, _P],
    "nekmesh_h1mg_levels": [_IP, _P],
    "nekmesh_face_types": [_IP, _IP, _P, _P, _P],
    "nekmesh_h1mg_level": [_IP, _IP, _P, _P, _P, _P, _P, _P, _IP, _IP, _P, _P, _P, _P],
    "nekmesh_fdm1d": [_IP, _IP, _IP, _DP, _DP, _DP, _P, _P],
    "nekmesh_xxt_factor": [_I64P, _P, _P, _P, _P, _I64P, _P, _P, _P, _P],
    "nekgpu_setup_xyz": [_I64P, _IP, _IP, _P, _P, _P, _P, _P, _P],
    "nekgpu_geom_update_dev": [_I64P, _P, _P, _P, _P],
    "nekgpu_geometry": [_I64P, _P, _P, _P, _P, _P, _P, _P],
    "nekgpu_gs_maps": [_I64P, _I64P, _I64P, _P, _P],
    "nekgpu_axhelm": [_I64P, _P, _P, _P, _P, _IP, _IP],
    "nekgpu_axhelm_dev": [_I64P, _P, _P, _P, _P, _IP, _IP],
    "nekgpu_axhelm_dev_noalloc": [_I64P, _P, _P, _P, _P, _IP, _IP],
    "nekgpu_dssum": [_I64P, _P],
    "nekgpu_dssum_dev": [_I64P, _P],
    "nekgpu_dsop_dev": [_I64P, _P, C.c_char_p],
    "nekgpu_setprec": [_I64P, _P, _P, _P, _IP, _IP],
    "nekgpu_setprec_dev": [_I64P, _P, _P, _P, _IP, _IP],
    "nekgpu_cggo": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP, _DP, _DP],
    "nekgpu_cggo_dev": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP, _DP, _DP],
    "nekgpu_hmholtz": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP, _DP, _DP],
    "nekgpu_hmholtz_dev": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP, _DP,
                           _DP],
    "nekgpu_set_timing": [_I64P, _IP],
    "nekgpu_last_timing": [_I64P, _DP, _DP, _IP],
    "nekgpu_launch_count": [_I64P],
    "nekgpu_autotune": [_I64P, _IP, _IP, _IP, _IP, _IP, _DP],
    "nekgpu_batch_shape": [_I64P, _IP, _IP, _DP],
    "nekgpu_batch_operator_forms": [_I64P, _IP],
    "nekgpu_last_kernel_times": [_I64P, _DP, _DP, _DP, _IP],
    "nekgpu_hsolve_dev": [_I64P, _IP, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP,
                          _DP, _DP, _IP],
    "nekgpu_hsolve": [_I64P, _IP, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP, _DP,
                      _DP, _IP],
    "nekgpu_proj_setup": [_I64P, _IP, _IP],
    "nekgpu_cggo_mixed_multi_dev": [_I64P, _IP, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P,
                                    _DP, _IP, _IP, _DP, _DP, _IP],
    "nekgpu_proj_count": [_I64P, _IP, _IP],
    "nekgpu_batch_set_shape": [_I64P, _IP, _IP],
    "nekgpu_batch_set_persistent": [_I64P, _IP],
    "nekgpu_crs_amg_setup": [_I64P, _I64P, _I64P, _P, _P, _P, _IP],
    "nekgpu_crs_amg_solve_dev": [_I64P, _P, _P],
    "nekgpu_ax_shape": [_I64P, _IP, _IP, _IP, _DP],
    "nekgpu_gs_shape": [_I64P, _IP, _IP, _IP, _DP],
    "nekgpu_set_gs_shape": [_I64P, _IP, _IP],
    "nekgpu_set_ax_shape": [_I64P, _IP, _IP, _IP],
    "nekgpu_ax_candidates": [_I64P, _IP, _P, _P, _IP],
    "nekgpu_cggo_mixed_dev": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _DP, _IP, _IP,
                              _DP, _DP],
    "nekgpu_hmholtz_mixed": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _DP, _IP, _IP,
                             _DP, _DP],
    "nekgpu_axhelm_adjoint_h1": [_I64P, _P, _P, _P],
    "nekgpu_axhelm_adjoint_h1_dev": [_I64P, _P, _P, _P],
    "nekgpu_cggo_adjoint_dev": [_I64P, _P, _P, _P, _P, _P, _P, _IP, _DP, _IP, _IP, _P, _IP, _IP, _DP,
                                _DP],
    "nekgpu_batch_create": [_IP, _I64P],
    "nekgpu_batch_add": [_I64P, _IP, _IP, _P, _P, _P, _P, _P, _P, _P, _P, _P, _IP],
    "nekgpu_batch_solve_dev": [_I64P, _IP, _P, _P, _P, _P, _P, _P, _P, _DP, _IP, _IP, _DP, _P, _P,
                               _P, _P, _P],
    "nekgpu_batch_last_error": [_I64P, C.c_char_p, _IP],
    "nekgpu_batch_destroy": [_I64P],
}

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return LIB_PATH


def load():
    """Load libnekgpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -m nek5000_gb300.build` "
                    "(nvcc, sm_103a); there is no CPU fallback")
            L = C.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = C.c_int
            _lib = L
    return _lib


class NekGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code
