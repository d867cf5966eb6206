"""ctypes binding of libuhs.so (include/uhs.h, include/uhs_dsl.h).

The library is the product: every call below goes straight to the C ABI.
Loading fails loudly when libuhs.so has not been built; there is no Python or
CPU fallback for any stencil operation.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libuhs.so")

# status codes (uhs.h)
UHS_OK, UHS_EINVAL, UHS_EUNSUPPORTED, UHS_ECUDA, UHS_ETIMEOUT, UHS_ENOMEM, UHS_ERANGE, UHS_EPARSE = range(8)
STATUS_NAMES = {0: "UHS_OK", 1: "UHS_EINVAL", 2: "UHS_EUNSUPPORTED", 3: "UHS_ECUDA", 4: "UHS_ETIMEOUT",
                5: "UHS_ENOMEM", 6: "UHS_ERANGE", 7: "UHS_EPARSE"}
# element types
UHS_F64, UHS_F32, UHS_F32X2 = 0, 1, 2
# arithmetic
UHS_ARITH_AUTO, UHS_ARITH_FMA, UHS_ARITH_EXACT, UHS_ARITH_DF32 = 0, 1, 2, 3
# kernel families
UHS_KERNEL_AUTO, UHS_KERNEL_GENERIC, UHS_KERNEL_STREAM, UHS_KERNEL_MMA = 0, 1, 2, 3
# flags
UHS_FLAG_NO_SYNC, UHS_FLAG_NO_TUNE_DB, UHS_FLAG_NO_FACTOR, UHS_FLAG_MMA_TMEM_A, UHS_FLAG_IN_PLACE = 1, 2, 4, 8, 16
UHS_FLAG_XSHUFFLE = 32

UHS_MAX_TERMS = 512
UHS_NOALLOC_MAX_PARTIALS = 8192
UHS_MAX_RADIUS = 4


class UhsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Memref(ctypes.Structure):
    _fields_ = [("allocated", c_void_p), ("aligned", c_void_p), ("offset", c_int64),
                ("sizes", c_int64 * 3), ("strides", c_int64 * 3)]


class Term(ctypes.Structure):
    _fields_ = [("dz", c_int32), ("dy", c_int32), ("dx", c_int32), ("param", c_int32), ("coef", c_double)]


class StencilDesc(ctypes.Structure):
    _fields_ = [("rank", c_int32), ("dtype", c_int32), ("lb", c_int64 * 3), ("ub", c_int64 * 3),
                ("nterms", c_int32), ("terms", POINTER(Term)), ("iterations", c_int32),
                ("params", POINTER(c_double)), ("nparams", c_int32)]


class Params(ctypes.Structure):
    _fields_ = [("kernel", c_int32), ("arith", c_int32), ("tile_x", c_int32), ("tile_y", c_int32),
                ("tile_z", c_int32), ("k_temporal", c_int32), ("use_tma", c_int32), ("flags", c_int32),
                ("vy", c_int32), ("prefetch", c_int32), ("factored", c_int32), ("vx", c_int32)]


# Every symbol include/*.h declares, with its ctypes signature: (restype, argtypes).
SIGNATURES = {
    "uhs_last_error": (c_char_p, []),
    "uhs_abi_version": (c_int, []),
    "uhs_params_default": (None, [POINTER(Params)]),
    "uhs_validate": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref)]),
    "uhs_run": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref), POINTER(Params), c_void_p]),
    "uhs_sweep": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref), POINTER(Params), c_void_p]),
    "uhs_plan": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Params), POINTER(Params)]),
    "uhs_launch_count": (c_int64, []),
    "uhs_launch_geometry": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Params), POINTER(c_int64)]),
    "uhs_release_scratch": (c_int, []),
    "uhs_probe_wait_timeout": (c_int, [c_int64, c_void_p]),
    "uhs_probe_dfma_rate": (c_int, [POINTER(c_double), c_void_p]),
    "uhs_set_alloc_cap": (c_int, [c_int64]),
    "uhs_tune_save": (c_int, [c_char_p]),
    "uhs_tune_load": (c_int, [c_char_p]),
    "uhs_mlp_create": (c_int, [c_int32, c_int32, c_int32, ctypes.c_uint64, POINTER(c_void_p)]),
    "uhs_mlp_destroy": (None, [c_void_p]),
    "uhs_mlp_num_params": (c_int64, [c_void_p]),
    "uhs_mlp_get_params": (c_int, [c_void_p, POINTER(ctypes.c_float)]),
    "uhs_mlp_set_params": (c_int, [c_void_p, POINTER(ctypes.c_float)]),
    "uhs_mlp_forward": (c_int, [c_void_p, POINTER(ctypes.c_float), c_int32, POINTER(ctypes.c_float)]),
    "uhs_mlp_loss_grad": (c_int, [c_void_p, POINTER(ctypes.c_float), POINTER(ctypes.c_float), c_int32,
                                  POINTER(ctypes.c_float), POINTER(ctypes.c_float)]),
    "uhs_mlp_train": (c_int, [c_void_p, POINTER(ctypes.c_float), POINTER(ctypes.c_float), c_int32, c_int32, c_int32,
                              ctypes.c_float, ctypes.c_uint64, POINTER(ctypes.c_float)]),
    "uhs_tune_put": (c_int, [POINTER(StencilDesc), POINTER(Params), c_double]),
    "uhs_tune_get": (c_int, [POINTER(StencilDesc), POINTER(Params), POINTER(c_int32)]),
    "uhs_tune_clear": (None, []),
    "uhs_tune_size": (c_int64, []),
    "uhs_batch_create": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref), c_int32, POINTER(Params),
                                 POINTER(c_void_p)]),
    "uhs_batch_run": (c_int, [c_void_p, c_void_p, c_int32]),
    "uhs_batch_stats": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    "uhs_batch_destroy": (None, [c_void_p]),
    "uhs_run_batch": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref), c_int32, POINTER(Params),
                              c_void_p]),
    "uhs_error_norms": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref), POINTER(c_double),
                                c_void_p]),
    "uhs_error_norms_noalloc": (c_int, [POINTER(StencilDesc), POINTER(Memref), POINTER(Memref),
                                        POINTER(c_double), c_void_p]),
    # uhs_dsl.h
    "uhs_dsl_parse": (c_int, [c_char_p, c_char_p, POINTER(c_void_p)]),
    "uhs_program_free": (None, [c_void_p]),
    "uhs_program_name": (c_char_p, [c_void_p]),
    "uhs_program_desc": (c_int, [c_void_p, POINTER(StencilDesc), POINTER(c_int64)]),
    "uhs_program_exact_order": (c_int, [c_void_p]),
    "uhs_program_tile": (c_int, [c_void_p, POINTER(c_int64)]),
    "uhs_program_num_kernels": (c_int, [c_void_p]),
    "uhs_program_num_param_arrays": (c_int, [c_void_p]),
    "uhs_program_set_params": (c_int, [c_void_p, POINTER(c_double), c_int32]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded libuhs.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                               f"g.build()\"` (or python uxxxxxxxxh_gb300/build.py)")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def last_error() -> str:
    return lib().uhs_last_error().decode()


def check(code: int) -> None:
    if code != UHS_OK:
        raise UhsError(code, last_error())
