"""ctypes binding of ``libellipticforest_gb300.so`` (the C ABI in ``include/ellipticforest_gb300.h``).

Loading never falls back to anything: if the library is missing or cannot be loaded, every entry
point of this package raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libellipticforest_gb300.so"

EF_OK = 0
EF_ERR_INVALID = -1
EF_ERR_CUDA = -2
EF_ERR_NOMEM = -3
EF_ERR_SINGULAR = -4
EF_ERR_STATE = -5
EF_ERR_UNSUPPORTED = -6

EF_SOLVER_FIVE_POINT = 0
EF_SOLVER_FISHPACK90 = 1

REFINE_FN = C.CFUNCTYPE(C.c_int, C.c_double, C.c_double, C.c_void_p)

_dp = C.POINTER(C.c_double)
_vp = C.c_void_p

# name -> (restype, argtypes); every function of the header
SIGNATURES = {
    "ef_last_error": (C.c_char_p, []),
    "ef_version": (C.c_int, []),
    "ef_mesh_create_refined": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                         C.c_int, C.c_int, REFINE_FN, _vp, C.POINTER(_vp)]),
    "ef_mesh_create_uniform": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                         C.c_int, C.POINTER(_vp)]),
    "ef_mesh_num_leaves": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "ef_mesh_num_nodes": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "ef_mesh_leaf": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_longlong),
                               C.POINTER(C.c_longlong), _dp]),
    "ef_mesh_destroy": (C.c_int, [_vp]),
    "ef_hps_create": (C.c_int, [_vp, C.c_int, C.c_double, C.POINTER(_vp)]),
    "ef_hps_set_coefficients": (C.c_int, [_vp, _dp, _dp, _dp]),
    "ef_hps_set_option": (C.c_int, [_vp, C.c_char_p, C.c_int]),
    "ef_hps_set_stream": (C.c_int, [_vp, _vp]),
    "ef_hps_info": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                              C.POINTER(C.c_longlong)]),
    "ef_hps_setup": (C.c_int, [_vp]),
    "ef_hps_build": (C.c_int, [_vp]),
    "ef_hps_upwards": (C.c_int, [_vp, _dp]),
    "ef_hps_solve": (C.c_int, [_vp, _dp, _dp, _dp]),
    "ef_hps_solve_root_dirichlet": (C.c_int, [_vp, _dp]),
    "ef_hps_get_leaf_u": (C.c_int, [_vp, _dp]),
    "ef_hps_get_root_T": (C.c_int, [_vp, _dp]),
    "ef_hps_get_root_h": (C.c_int, [_vp, _dp]),
    "ef_hps_destroy": (C.c_int, [_vp]),
    "ef_hps_device_buffers": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                        C.POINTER(_vp), C.POINTER(_vp)]),
    "ef_hps_load_device_async": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "ef_hps_solve_device_async": (C.c_int, [_vp, C.c_int]),
    "ef_hps_synchronize": (C.c_int, [_vp]),
    "ef_hps_mixed_init": (C.c_int, [_vp, C.c_int]),
    "ef_hps_mixed_buffers": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    "ef_hps_mixed_solve_async": (C.c_int, [_vp, C.c_int, C.c_int]),
    "ef_hps_mixed_solve": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp, _dp, _dp]),
    "ef_hps_mixed_residuals": (C.c_int, [_vp, C.c_int, _dp]),
    "ef_hps_build_mixed": (C.c_int, [_vp, C.c_int]),
    "ef_hps_root_factorizations": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "ef_hps_save": (C.c_int, [_vp, C.c_char_p]),
    "ef_hps_build_from": (C.c_int, [_vp, _vp, C.POINTER(C.c_int)]),
    "ef_hps_load": (C.c_int, [C.c_char_p, C.POINTER(_vp), C.POINTER(_vp)]),
    "ef_server_create": (C.c_int, [C.POINTER(_vp), C.POINTER(C.c_int), C.c_int, C.c_int, C.c_longlong, C.c_int,
                                   C.POINTER(_vp)]),
    "ef_server_info": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "ef_server_set_sweeps": (C.c_int, [_vp, C.c_int, C.c_int]),
    "ef_hps_mixed_lane": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "ef_hps_mixed_lane_solve_async": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    "ef_hps_mixed_solve_blocks": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_void_p),
                                            C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "ef_server_submit": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(C.c_longlong)]),
    "ef_server_poll": (C.c_int, [_vp, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "ef_server_wait": (C.c_int, [_vp, C.c_longlong, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "ef_server_stats": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_longlong)]),
    "ef_server_destroy": (C.c_int, [_vp]),
    "ef_kernel_launches": (C.c_int, [C.POINTER(C.c_longlong)]),
    "ef_hps_profile_enable": (C.c_int, [_vp, C.c_int]),
    "ef_hps_profile_count": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "ef_hps_profile_entry": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int, _dp, C.POINTER(C.c_longlong),
                                       C.POINTER(C.c_longlong), _dp, _dp]),
    "ef_hps_profile_reset": (C.c_int, [_vp]),
    "ef_fv_build_d2n": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                  C.c_double, _dp]),
    "ef_fv_solve": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                              _dp, _dp, _dp]),
    "ef_fv_map_d2n": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, _dp, _dp, _dp]),
    "ef_fv5_build_d2n": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp]),
    "ef_fv5_solve": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp,
                               _dp]),
    "ef_fv5_map_d2n": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp,
                                 _dp, _dp]),
    "ef_hps_build_info": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "ef_hps_mixed_gemm_plan": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ef_hps_mixed_set_gemm_plan": (C.c_int, [_vp, C.POINTER(C.c_int), C.c_int]),
    "ef_hps_mixed_set_root": (C.c_int, [_vp, _dp, _dp]),
    "ef_server_set_root": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "ef_mesh_level_count": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "ef_mesh_subtree": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "ef_hps_split_sizes": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "ef_hps_build_top": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "ef_hps_upwards_top": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "ef_hps_solve_top": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, C.POINTER(_vp)]),
    "ef_fv_solve_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_double, _vp, _vp, _vp, _vp]),
}

_LIB = None


class EFError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ellipticforest_gb300 error {code}: {msg}")
        self.code = code


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load (once) and return the library; raises RuntimeError when it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python -m ellipticforest_gb300.build). "
            "There is no CPU fallback.")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(code: int) -> int:
    if code != EF_OK:
        msg = load().ef_last_error()
        raise EFError(code, msg.decode() if msg else "")
    return code


def dptr(a) -> "C.POINTER(C.c_double)":
    return a.ctypes.data_as(_dp)
