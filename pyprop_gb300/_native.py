"""ctypes binding of libpyprop_gpu.so (the C ABI declared in include/pyprop_gpu.h).

The library is the only compute path: if it is missing or no CUDA device is present the
calls raise, they never fall back to host code.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpyprop_gpu.so")

PG_OK = 0
PG_FP64 = 0
PG_FP32 = 1

PG_BAND_MUL_U = 0
PG_BAND_MUL_UT = 1
PG_BAND_SOLVE_U = 2
PG_BAND_SOLVE_UT = 3
PG_BAND_MUL_S = 4
PG_BAND_SOLVE_S = 5
PG_BAND_PREC_SOLVE = 6
PG_ERR_STORAGE = -3
PG_ERR_SHAPE = -4
PG_ERR_NOT_CONVERGED = -7
PG_ERR_STATE = -9

ERRORS = {
    -1: "PG_ERR_ARG", -2: "PG_ERR_CUDA", -3: "PG_ERR_STORAGE", -4: "PG_ERR_SHAPE", -5: "PG_ERR_NONFINITE",
    -6: "PG_ERR_BREAKDOWN", -7: "PG_ERR_NOT_CONVERGED", -8: "PG_ERR_ALLOC", -9: "PG_ERR_STATE",
}


class PygpuError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        msg = _lib.pg_error_string(code).decode() if _lib is not None else ERRORS.get(code, str(code))
        super().__init__("%s failed: %s (%d)" % (where, msg, code))


class KrylovStats(C.Structure):
    _fields_ = [("OpCount", C.c_longlong), ("InnerProductCount", C.c_longlong), ("ReOrthoCount", C.c_longlong),
                ("RestartCount", C.c_longlong), ("Iterations", C.c_longlong), ("ErrorEstimate", C.c_double),
                ("TrueResidual", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_LL = C.c_longlong
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_SIGS = {
    "pg_error_string": (C.c_char_p, [_I]),
    "pg_version": (C.c_char_p, []),
    "pg_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "pg_ctx_destroy": (_I, [_P]),
    "pg_ctx_stream": (_P, [_P]),
    "pg_ctx_set_stream": (_I, [_P, _P]),
    "pg_ctx_use_own_stream": (_I, [_P]),
    "pg_ctx_kernel_launches": (_LL, [_P]),
    "pg_ctx_synchronize": (_I, [_P]),
    "pg_ctx_device_error": (_I, [_P, _IP]),
    "pg_ctx_clear_device_error": (_I, [_P]),
    "pg_tensor_multiply_diag_bandnh": (_I, [_P, _I, _I, _D, _P, _I, _I, _P, _I, _I, _I, _P]),
    "pg_tensor_multiply_simp_bandnh": (_I, [_P, _I, _I, _D, _P, _I, _I, _P, _I, _I, _P, _I, _I, _I, _P]),
    "pg_tensor_multiply_ident_bandnh": (_I, [_P, _I, _I, _D, _P, _I, _I, _P, _I, _I, _I, _P]),
    "pg_op_create": (_I, [_P, _I, _IP, _I, _I, C.POINTER(_P)]),
    "pg_op_destroy": (_I, [_P]),
    "pg_op_add_term": (_I, [_P, C.c_char_p, _DP, _I, _I, _IP, _I, _I]),
    "pg_op_add_term_ranks": (_I, [_P, C.c_char_p, _DP, _IP, _IP, _IP, _I]),
    "pg_op_finalize": (_I, [_P]),
    "pg_op_variant": (_I, [_P, _I, _IP, C.POINTER(C.c_float)]),
    "pg_op_stored_elements": (_LL, [_P]),
    "pg_prec_fd_create": (_I, [_P, _I, _DP, _DP, _IP, _DP, _DP, C.POINTER(_P)]),
    "pg_prec_fd_max_n": (_I, [_I]),
    "pg_pamp_batch_create": (_I, [C.POINTER(_P), _I, C.POINTER(_P)]),
    "pg_pamp_batch_destroy": (_I, [_P]),
    "pg_pamp_batch_step": (_I, [_P, C.POINTER(_P), _D, _DP, _I]),
    "pg_pamp_batch_stats": (_I, [_P, C.POINTER(KrylovStats)]),
    "pg_pamp_batch_set_mode": (_I, [_P, _I]),
    "pg_pamp_batch_get_mode": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float)]),
    "pg_op_add_factored": (_I, [_P, _I, _DP, _DP, _IP, _LL, _IP, _IP, _IP, _DP]),
    "pg_op_factored_info": (_I, [_P, _DP]),
    "pg_op_set_fp64_emulation": (_I, [_P, _I]),
    "pg_op_matvec": (_I, [_P, _DP, _I, _P, _P, _I]),
    "pg_overlap_create": (_I, [_P, _DP, C.POINTER(_P)]),
    "pg_prec_blockdiag_create": (_I, [_P, _DP, _DP, _DP, _IP, _DP, _I, C.POINTER(_P)]),
    "pg_banded_destroy": (_I, [_P]),
    "pg_banded_apply": (_I, [_P, _I, _P]),
    "pg_pamp_create": (_I, [_P, _P, _P, _P, _I, _I, _I, C.POINTER(_P)]),
    "pg_pamp_destroy": (_I, [_P]),
    "pg_pamp_step": (_I, [_P, _P, _D, _DP, _I, C.POINTER(KrylovStats)]),
    "pg_pamp_set_device_exp": (_I, [_P, _I]),
    "pg_pamp_last_stats": (_I, [_P, C.POINTER(KrylovStats)]),
    "pg_pamp_set_fused": (_I, [_P, _I]),
    "pg_pamp_set_barrier_probe": (_I, [_P, _I, _I]),
    "pg_cayley_create": (_I, [_P, _P, _P, _P, _I, _I, _D, C.POINTER(_P)]),
    "pg_cayley_destroy": (_I, [_P]),
    "pg_cayley_step": (_I, [_P, _P, _D, _DP, _I, C.POINTER(KrylovStats)]),
    "pg_cayley_advance": (_I, [_P, _P, _D, _I, _DP, _I, C.POINTER(KrylovStats)]),
    "pg_cayley_last_stats": (_I, [_P, C.POINTER(KrylovStats)]),
    "pg_cayley_set_true_residual": (_I, [_P, _I]),
    "pg_cayley_set_eager": (_I, [_P, _I]),
    "pg_cayley_set_fused": (_I, [_P, _I]),
    "pg_cayley_set_barrier_probe": (_I, [_P, _I, _I]),
    "pg_cayley_totals": (_I, [_P, C.POINTER(_LL), C.POINTER(_LL)]),
    "pg_cayley_set_fused_variant": (_I, [_P, _I]),
    "pg_cayley_get_fused_variant": (_I, [_P, _IP]),
    "pg_cayley_set_learned": (_I, [_P, _P, _I]),
    "pg_cayley_learned_rejected": (_I, [_P, C.POINTER(_LL)]),
    "pg_cayley_batch_create": (_I, [C.POINTER(_P), _I, C.POINTER(_P)]),
    "pg_cayley_batch_destroy": (_I, [_P]),
    "pg_cayley_batch_step": (_I, [_P, C.POINTER(_P), _D, _DP, _I]),
    "pg_cayley_batch_stats": (_I, [_P, C.POINTER(KrylovStats)]),
    "pg_arnoldi_expand": (_I, [_P, _P, _P, _DP, _I, _P, _I, _I, _P, _DP, _D, _I, _IP, _DP,
                               C.POINTER(KrylovStats)]),
    "pg_vec_dot": (_I, [_P, _I, _P, _P, _LL, _DP]),
    "pg_vec_convert": (_I, [_P, _I, _P, _I, _P, _LL]),
    "pg_vec_combine": (_I, [_P, _P, _LL, _I, _DP, _I]),
    "pg_vec_swap_last2": (_I, [_P, _I, _P, _P, _I, _I, _I]),
    "pg_prec_kron_create": (_I, [_P, _DP, _DP, _DP, _DP, _DP, C.POINTER(_P)]),
    "pg_mlp_create": (_I, [_P, _I, _I, _I, C.c_ulonglong, C.POINTER(_P)]),
    "pg_mlp_destroy": (_I, [_P]),
    "pg_mlp_parameter_count": (_LL, [_P]),
    "pg_mlp_get_weights": (_I, [_P, _P]),
    "pg_mlp_set_weights": (_I, [_P, _P]),
    "pg_mlp_forward": (_I, [_P, _P, _I, _P]),
    "pg_mlp_gradients": (_I, [_P, _P, _P, _I, _DP, _P]),
    "pg_mlp_train_step": (_I, [_P, _P, _P, _I, C.c_float, _DP]),
    "pg_mlp_block_features": (_I, [_P, _P, _I, _I, _I, _P]),
    "pg_vec_multidot_noalloc": (_I, [_I, _P, _LL, _I, _P, _LL, _P, _P]),
    "pg_bspline_band_project": (_I, [_P, _P, _LL, _I, _LL, _LL, _I, _I, _I, _P, _P, _P, _I, _P, _LL, _LL, _LL,
                                     _LL]),
    "pg_radial_products_project": (_I, [_P, _P, _I, _I, _I, _IP, _I, _DP, _I, _DP, _I, _DP]),
    "pg_radial_products_remove": (_I, [_P, _P, _P, _I, _I, _I, _IP, _I, _DP, _I, _DP, _I]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols():
    """Names the binding expects the library to export."""
    return sorted(_SIGS)


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH) or build_if_missing:
            from . import build_native
            try:
                build_native.build()
            except Exception:
                if not os.path.exists(LIB_PATH):
                    raise
        if not os.path.exists(LIB_PATH):
            raise ImportError("libpyprop_gpu.so is not built (run pyprop_gb300.build_native)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(code, where):
    if code != PG_OK:
        raise PygpuError(code, where)
    return code


def dptr(arr):
    """ctypes double* for a contiguous numpy float64/complex128 array."""
    import numpy as np
    a = np.ascontiguousarray(arr)
    return a, a.ctypes.data_as(_DP)


def iptr(arr):
    import numpy as np
    a = np.ascontiguousarray(arr, dtype=np.int32)
    return a, a.ctypes.data_as(_IP)
