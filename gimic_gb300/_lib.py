"""ctypes binding of libgimic_gb300.so (declarations in include/gimic_gb300.h).

The library is built in-tree by ``gimic_gb300.build``; a missing library is an
error (there is no CPU fallback for the evaluation path).
"""
import ctypes as C
import os

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None

GG_OK = 0
GG_PREC_FP64 = 0
GG_PREC_SPLIT16 = 1
_ERRORS = {-1: "EINVAL", -2: "EIO", -3: "ECUDA", -4: "ENOMEM", -5: "ETIMEDOUT", -6: "EUNSUPPORTED"}


class GridSpec(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("basv", C.c_double * 9), ("npts", C.c_int * 3),
                ("pts", _dp * 3), ("wgt", _dp * 3), ("radius", C.c_double)]


# name -> (restype, argtypes) for every symbol declared in include/gimic_gb300.h
SIGNATURES = {
    "gimic_init": (None, [C.c_char_p, C.c_char_p]),
    "gimic_finalize": (None, []),
    "gimic_set_uhf": (None, [_ip]),
    "gimic_set_magnet": (None, [_dp]),
    "gimic_set_spin": (None, [C.c_char_p]),
    "gimic_set_screening": (None, [_dp]),
    "gimic_calc_jtensor": (None, [_dp, _dp]),
    "gimic_calc_jvector": (None, [_dp, _dp]),
    "gimic_calc_modj": (None, [_dp, _dp]),
    "gimic_get_gauss_points": (None, [_dp, _dp, _ip, _ip, _dp, _dp]),
    "mkgausspoints": (None, [_dp, _dp, _ip, _ip, _dp, _dp]),
    "gg_ctx_create": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.POINTER(C.c_void_p)]),
    "gg_ctx_create_ex": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.c_int,
                                   C.POINTER(C.c_void_p)]),
    "gg_spherical_projection": (C.c_int, [C.c_int, _dp]),
    "gg_ctx_destroy": (C.c_int, [C.c_void_p]),
    "gg_last_error": (C.c_char_p, [C.c_void_p]),
    "gg_set_spin": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gg_set_magnet": (C.c_int, [C.c_void_p, _dp]),
    "gg_get_magnet": (C.c_int, [C.c_void_p, _dp]),
    "gg_set_screening": (C.c_int, [C.c_void_p, C.c_double]),
    "gg_set_flags": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "gg_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_set_max_batch": (C.c_int, [C.c_void_p, C.c_int64]),
    "gg_set_tile_screening": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_set_cross_skip": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_set_shell_order": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_get_shell_order": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gg_basis_info": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip]),
    "gg_atoms": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gg_jtensor_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "gg_jvector_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "gg_plane_integral": (C.c_int, [C.c_void_p, C.POINTER(GridSpec), _dp, C.c_void_p]),
    "gg_plane_integrals": (C.c_int, [C.c_void_p, C.POINTER(GridSpec), C.c_int, _dp, C.c_void_p]),
    "gg_plane_integrals_enqueue": (C.c_int, [C.c_void_p, C.POINTER(GridSpec), C.c_int, C.c_void_p]),
    "gg_plane_integrals_collect": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gg_gauss_data": (C.c_int, [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    "gg_au2si": (C.c_double, [C.c_double]),
    "gg_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_profile_blocks": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gg_plane_integrals_batch": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(C.POINTER(GridSpec)), _ip, C.c_int,
                                           C.c_int, _dp, _dp, C.c_void_p]),
    "gg_selftest_wait_timeout": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.c_void_p]),
    "gg_selftest_fail_next": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_jtensor_batch_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p]),
    "gg_profile_read": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gg_profile_cross": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "gg_jtensor_batch_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "gg_properties": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, _dp, C.c_int, C.POINTER(C.c_int64), C.c_int, _dp,
                                _dp, C.c_void_p]),
    "gg_mlp_nparams": (C.c_int, []),
    "gg_mlp_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "gg_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gg_mlp_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float,
                              C.c_float, C.c_int, C.c_void_p]),
    "gg_mlp_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
}


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) and declare every exported symbol."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libgimic_gb300.so is missing; run gimic_gb300.build.build()")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class GimicError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%s)" % (msg, _ERRORS.get(code, code)))
        self.code = code


def check(rc, ctx=None):
    if rc != GG_OK:
        msg = load().gg_last_error(ctx)
        raise GimicError(rc, msg.decode() if msg else "error")
