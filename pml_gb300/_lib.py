"""ctypes binding of libpmlg.so (the C ABI declared in include/pmlg.h).

Importing this module loads the in-tree CUDA library and raises if it is
missing: there is no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libpmlg.so"

PMLG_OK = 0
STATUS = {0: "PMLG_OK", 1: "PMLG_EINVAL", 2: "PMLG_EBADMOD", 3: "PMLG_ENOROOT", 4: "PMLG_ELEN",
          5: "PMLG_EALIAS", 6: "PMLG_ETIMEOUT", 7: "PMLG_ECUDA", 8: "PMLG_ENOMEM", 9: "PMLG_EUNSUP"}
FORM_AUTO, FORM_CUDA_CORE, FORM_INT8_TC, FORM_F16_TC = 0, 1, 2, 3

_vp = C.c_void_p
_i64 = C.c_int64
_u64 = C.c_uint64
_i64p = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every entry point of include/pmlg.h
SIGNATURES = {
    "pmlg_ctx_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "pmlg_ctx_destroy": (C.c_int, [_vp]),
    "pmlg_ctx_set_form": (C.c_int, [_vp, C.c_int]),
    "pmlg_ctx_set_leaf_order": (C.c_int, [_vp, _i64]),
    "pmlg_ctx_set_tuning": (C.c_int, [_vp, C.c_int]),
    "pmlg_ctx_tuned_form": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _i64]),
    "pmlg_ctx_set_batch_graphs": (C.c_int, [_vp, C.c_int]),
    "pmlg_ctx_launch_count": (C.c_ulonglong, [_vp]),
    "pmlg_ctx_last_error": (C.c_char_p, [_vp]),
    "pmlg_ctx_device_status": (C.c_int, [_vp, _vp]),
    "pmlg_ctx_selftest_timeout": (C.c_int, [_vp, C.c_ulonglong, _vp]),
    "pmlg_ctx_set_profiling": (C.c_int, [_vp, C.c_int]),
    "pmlg_ctx_profile_read": (C.c_int, [_vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_double),
                                        C.POINTER(C.c_ulonglong), C.c_int, C.POINTER(C.c_int)]),
    "pmlg_strerror": (C.c_char_p, [C.c_int]),
    "pmlg_nmod_mat_mul_batch_u32": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _u64, _vp]),
    "pmlg_poly_mat_mul": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _u64, _vp]),
    "pmlg_poly_mat_mulmid": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _i64, _i64, _u64,
                                       _i64p, _vp]),
    "pmlg_poly_mat_mul_host": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _u64, _vp]),
    "pmlg_poly_mat_mulmid_host": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _i64, _i64,
                                            _u64, _i64p, _vp]),
    "pmlg_poly_mat_mul_batch": (C.c_int, [_vp, _vp, _i64, _vp]),
    "pmlg_pmbasis": (C.c_int, [_vp, _vp, _i64, _i64p, _vp, _i64, _i64, _i64, _i64, _u64, _i64p, _vp]),
    "pmlg_mbasis": (C.c_int, [_vp, _vp, _i64, _i64p, _vp, _i64, _i64, _i64, _i64, _u64, _i64p, _vp]),
    "pmlg_pmbasis_host": (C.c_int, [_vp, _vp, _i64, _i64p, _vp, _i64, _i64, _i64, _i64, _u64, _i64p, _vp]),
    "pmlg_kernel_via_approx": (C.c_int, [_vp, _vp, _i64, _i64p, _i64p, _i64p, _vp, _i64, _i64, _i64, _u64, _i64p,
                                         _vp]),
    "pmlg_kernel": (C.c_int, [_vp, _vp, _i64, _i64p, _i64p, _i64p, _vp, _i64, _i64, _i64, _u64, C.c_int, C.c_int,
                              _i64p, _vp]),
    "pmlg_popov_pmbasis": (C.c_int, [_vp, _vp, _i64, _i64p, _vp, _i64, _i64, _i64, _i64, _u64, _i64p, _vp]),
    "pmlg_kernel_zls": (C.c_int, [_vp, _vp, _i64, _i64p, _i64p, _i64p, _vp, _i64, _i64, _i64, _u64, _i64p, _vp]),
    "pmlg_kernel_zls_host": (C.c_int, [_vp, _vp, _i64, _i64p, _i64p, _i64p, _vp, _i64, _i64, _i64, _u64, _i64p,
                                       _vp]),
    "pmlg_inv_trunc": (C.c_int, [_vp, _vp, _vp, _i64, _i64, _i64, _u64, C.POINTER(C.c_int), _vp]),
    "pmlg_dixon": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _i64, _u64,
                             C.POINTER(C.c_int), _vp]),
    "pmlg_poly_mat_to_mat_poly": (C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _i64, _i64p, _vp]),
    "pmlg_mat_poly_to_poly_mat": (C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp]),
    "pmlg_nmod_vec_dot": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _u64, _vp]),
    "pmlg_nmod32_vec_dot": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _u64, _vp]),
    "pmlg_nmod32_vec_mdot": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _u64, _vp]),
    "pmlg_nmod_vec_dot_multi": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _i64, _u64, _vp]),
    "pmlg_nmod_vec_dot_multi_noalloc": (C.c_int, [_vp, _vp, _vp, _i64, _i64, _u64, _vp]),
    "pmlg_multimod_reduce": (C.c_int, [_vp, _vp, _vp, _i64, _vp, C.c_int, _vp]),
    "pmlg_multimod_crt": (C.c_int, [_vp, _vp, _vp, _i64, _vp, C.c_int, _u64, _vp]),
}


class PolymatJob(C.Structure):
    """pmlg_polymat_job"""
    _fields_ = [("r", _i64), ("k", _i64), ("c", _i64), ("len1", _i64), ("len2", _i64), ("p", _u64),
                ("A", _vp), ("B", _vp), ("C", _vp)]


class PmlgError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


_lib = None


def load() -> C.CDLL:
    """Loads libpmlg.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import _build
    if _build.needs_build():
        _build.build()
    if not LIB_PATH.exists():
        raise ImportError(f"libpmlg.so is missing at {LIB_PATH}: the CUDA library was not built")
    L = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int, ctx=None) -> None:
    if status != PMLG_OK:
        msg = ""
        if ctx is not None:
            msg = (load().pmlg_ctx_last_error(ctx) or b"").decode(errors="replace")
        raise PmlgError(status, msg)
