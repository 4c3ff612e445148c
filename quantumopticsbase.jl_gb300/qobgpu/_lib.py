"""ctypes binding of libqobgpu.so (declared in include/qobgpu.h).

There is no fallback: if the library is missing the import of the device layer
fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# QOB_LIBRARY selects another build of the same library (the bounds-checked
# build, libqobgpu_debug.so, for its own tests)
LIB_PATH = os.environ.get("QOB_LIBRARY") or os.path.join(_HERE, "libqobgpu.so")
ALLOC_HOOK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_size_t)

QOB_OK = 0
QOB_ERR_DIM = 1
QOB_ERR_ALIAS = 2
QOB_ERR_UNSUPPORTED = 3
QOB_ERR_ARG = 4
QOB_ERR_CUDA = 5
QOB_ERR_OOM = 6
QOB_ERR_TIMEOUT = 7
QOB_ERR_STATE = 8
QOB_ERR_CANCELLED = 9
QOB_C128 = 0
QOB_C64 = 1
QOB_C128X = 2  # ComplexF64 data, fused part in double-float arithmetic
QOB_OPT_FP64_TENSOR = 1
QOB_OPT_PDL = 2
QOB_OPT_FP32_TENSOR = 3
QOB_LEFT = 0
QOB_RIGHT = 1

VP = C.c_void_p
I64 = C.c_int64
I64P = C.POINTER(C.c_int64)
DP = C.POINTER(C.c_double)
D = C.c_double
I = C.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "qob_version": (I, []),
    "qob_kernel_launches": (I64, []),
    "qob_create": (I, [C.POINTER(VP), I, C.c_uint]),
    "qob_destroy": (I, [VP]),
    "qob_last_error": (C.c_char_p, [VP]),
    "qob_probe_peak": (I, [VP, I, DP]),
    "qob_probe_peak_ex": (I, [VP, I, DP, DP, DP]),
    "qob_set_option": (I, [VP, I, I64]),
    "qob_op_sparse": (I, [VP, I64, I64, I64P, I64P, VP, I, I, C.POINTER(VP)]),
    "qob_op_dense": (I, [VP, I64, I64, VP, I64, I, I, C.POINTER(VP)]),
    "qob_op_eye": (I, [VP, I64, I64, C.POINTER(VP)]),
    "qob_op_lazytensor": (I, [VP, I, I64P, I64P, I, I64P, C.POINTER(VP), D, D, C.POINTER(VP)]),
    "qob_op_lazysum": (I, [VP, I64, I64, I, DP, C.POINTER(VP), C.POINTER(VP)]),
    "qob_op_lazyproduct": (I, [VP, I, C.POINTER(VP), D, D, C.POINTER(VP)]),
    "qob_op_set_factors": (I, [VP, VP, DP]),
    "qob_op_free": (I, [VP, VP]),
    "qob_op_shape": (I, [VP, VP, I64P, I64P]),
    "qob_op_prepare": (I, [VP, VP, I, I, I64P]),
    "qob_op_tune": (I, [VP, VP, I, I, I64, DP, C.POINTER(C.c_int)]),
    "qob_op_tune_ex": (I, [VP, VP, I, I, I64, DP, I, C.POINTER(C.c_int)]),
    "qob_op_set_launch": (I, [VP, VP, I, I, I, I, I]),
    "qob_op_set_tile": (I, [VP, VP, I, I, I, I, I]),
    "qob_op_set_pairs": (I, [VP, VP, I, I, I, I, I]),
    "qob_device_status": (I, [VP, VP, C.POINTER(C.c_uint)]),
    "qob_mul": (I, [VP, I, I, VP, I, D, D, VP, I64, I64, I64, D, D, VP, I64, I64, I64, VP]),
    "qob_mul_host": (I, [VP, I, I, VP, I, D, D, VP, I64, I64, D, D, VP, I64, I64]),
    "qob_mul_host_async": (I, [VP, I, I, VP, I, D, D, VP, I64, I64, D, D, VP, I64, I64, VP]),
    "qob_host_wait": (I, [VP, C.c_uint64]),
    "qob_norm": (I, [VP, I, VP, I64, DP, VP]),
    "qob_dot": (I, [VP, I, VP, VP, I64, DP, VP]),
    "qob_expect": (I, [VP, VP, I, VP, I64, DP, VP]),
    "qob_variance": (I, [VP, VP, I, VP, I64, DP, VP]),
    "qob_expect_dm": (I, [VP, VP, I, VP, I64, I64, DP, VP]),
    "qob_dot_noalloc": (I, [VP, I, VP, VP, I64, VP, VP]),
    "qob_batch_create": (I, [VP, I, C.POINTER(VP)]),
    "qob_batch_add": (I, [VP, VP, VP, D, D, VP, VP, D, D]),
    "qob_batch_run": (I, [VP, VP, VP]),
    "qob_batch_tune": (I, [VP, VP, DP, C.POINTER(C.c_int)]),
    "qob_batch_info": (I, [VP, VP, I64P]),
    "qob_batch_set_tile": (I, [VP, VP, I]),
    "qob_batch_free": (I, [VP, VP]),
    "qob_rk4": (I, [VP, VP, I, VP, I64, D, I, I, VP]),
    "qob_apply_batched": (I, [VP, I, I, C.POINTER(VP), C.POINTER(VP), C.POINTER(VP), DP, DP, VP]),
    "qob_state_alloc": (I, [VP, I, I64, I64, C.POINTER(VP)]),
    "qob_state_free": (I, [VP, VP]),
    "qob_state_upload": (I, [VP, I, VP, VP, I64, I64, VP]),
    "qob_state_download": (I, [VP, I, VP, VP, I64, I64, VP]),
    "qob_op_fft": (I, [VP, I, I64P, I, I64P, C.POINTER(C.c_int), DP, DP, C.POINTER(VP)]),
    "qob_expect_lazyket": (I, [VP, VP, I, I, I64P, VP, I64, VP, VP]),
    "qob_rk4_td": (I, [VP, VP, I, VP, I64, D, I, VP, I64, I, VP]),
    "qob_server_create": (I, [VP, I, C.c_size_t, I, I, C.POINTER(VP)]),
    "qob_server_submit": (I, [VP, VP, VP, I64, I, D, I64P]),
    "qob_server_submit_td": (I, [VP, VP, VP, I64, I, D, VP, I64, I64P]),
    "qob_server_step": (I, [VP, C.POINTER(C.c_int)]),
    "qob_server_start": (I, [VP]),
    "qob_server_stop": (I, [VP]),
    "qob_server_poll": (I, [VP, I64, VP, DP, C.POINTER(C.c_int)]),
    "qob_server_wait": (I, [VP, I64, D, C.POINTER(C.c_int)]),
    "qob_server_stats": (I, [VP, I64P]),
    "qob_server_stats2": (I, [VP, I64P]),
    "qob_server_cancel": (I, [VP, I64]),
    "qob_server_set_alloc_hook": (I, [VP, VP, VP]),
    "qob_server_destroy": (I, [VP]),
    "qob_graph_begin": (I, [VP, VP]),
    "qob_graph_end": (I, [VP, VP, C.POINTER(VP)]),
    "qob_graph_launch": (I, [VP, VP, VP]),
    "qob_graph_free": (I, [VP, VP]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(nvcc, sm_103a). There is no CPU fallback."
            )
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(SIGNATURES)
