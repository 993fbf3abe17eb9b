"""ctypes binding of libadtomo_gpu.so (the C ABI in include/adtomo_gpu.h)."""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libadtomo_gpu.so")
_lock = threading.Lock()
_lib = None

ADT_OK = 0
ERRORS = {
    -1: "ADT_EINVAL",
    -2: "ADT_ENOMEM",
    -3: "ADT_ECUDA",
    -4: "ADT_ETIMEOUT",
    -5: "ADT_ENOCONV",
    -6: "ADT_ESINGULAR",
    -7: "ADT_ENODEV",
}
ADT_F32, ADT_F64 = 0, 1
ADT_ADJ_SWEEPS, ADT_ADJ_CAUSAL, ADT_ADJ_AUTO = 0, 1, 2


class AdtError(RuntimeError):
    """A negative return code of the library, with its message."""

    def __init__(self, code: int, message: str):
        self.code = code
        self.name = ERRORS.get(code, str(code))
        super().__init__(f"{self.name}: {message}")


class SolveStatus(C.Structure):
    _fields_ = [("iters", C.c_int32), ("converged", C.c_int32), ("final_err", C.c_double),
                ("adj_iters", C.c_int32), ("adj_converged", C.c_int32)]


class BatchOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("tol", C.c_double), ("max_iter", C.c_int32),
                ("adj_max_iter", C.c_int32), ("ref_compat", C.c_int32),
                ("near_src_f64", C.c_int32), ("chunk", C.c_int32), ("bk", C.c_int32),
                ("warps", C.c_int32), ("groups", C.c_int32), ("use_graph", C.c_int32),
                ("wake_tol", C.c_double), ("adj_wake_tol", C.c_double),
                ("adj_order_filter", C.c_int32), ("fwd_order_filter", C.c_int32),
                ("overlap_chunks", C.c_int32), ("adj_warps", C.c_int32),
                ("adj_groups", C.c_int32), ("adj_solver", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("fwd_cell_updates", C.c_int64), ("adj_cell_updates", C.c_int64),
                ("fwd_bricks", C.c_int64), ("adj_bricks", C.c_int64), ("fwd_ms", C.c_float),
                ("adj_ms", C.c_float), ("total_ms", C.c_float), ("bk", C.c_int32),
                ("warps", C.c_int32), ("groups", C.c_int32), ("ctas", C.c_int32),
                ("adj_warps", C.c_int32), ("adj_groups", C.c_int32), ("adj_solver", C.c_int32)]


_P = C.c_void_p
_D = C.c_double
_I64 = C.c_int64
_I32 = C.c_int32

# name -> (restype, argtypes); every symbol declared in include/adtomo_gpu.h
SIGNATURES = {
    "adt_last_error": (C.c_char_p, []),
    "adt_version": (C.c_char_p, []),
    "adt_device_count": (C.c_int, []),
    "adt_eikonal": (C.c_int, [_P, _I64, _I64, _I64, _I64, _D, _P, _P]),
    "adt_eikonal_grad": (C.c_int, [_P, _P, _P, _I64, _I64, _I64, _I64, _D, _P]),
    "adt_eikonal_batch": (C.c_int, [_P, _I64, _I64, _I64, _P, _P, _D, _P, _P]),
    "adt_eikonal_three_d": (C.c_int, [_P, _P, _D, _I64, _I64, _I64, _D, C.c_int, _P, _P]),
    "adt_eikonal_three_d_grad": (C.c_int, [_P, _P, _P, _P, _D, _I64, _I64, _I64, _D, C.c_int, _P,
                                           _P]),
    "adt_eikonal_three_d_device": (C.c_int, [_P, _P, _D, _I64, _I64, _I64, _D, C.c_int, _P, _P,
                                             _P]),
    "adt_eikonal_three_d_grad_device": (C.c_int, [_P, _P, _P, _P, _D, _I64, _I64, _I64, _P, _P,
                                                  _P]),
    "adt_eikonal_three_d_device_noalloc": (C.c_int, [_P, _P, _D, _I64, _I64, _I64, _D, C.c_int,
                                                     _P, _P, _P]),
    "adt_abi_struct_sizes": (C.c_int, [_P, _I32]),
    "adt_tile_layout": (C.c_int, [_I32, _P]),
    "adt_batch_opts_default": (None, [_P]),
    "adt_batch_create": (C.c_int, [_P, _I32, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "adt_batch_destroy": (C.c_int, [_P]),
    "adt_batch_run": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "adt_batch_upload": (C.c_int, [_P, _P, _P, _P]),
    "adt_batch_set_source_velocity": (C.c_int, [_P, _P]),
    "adt_batch_autotune": (C.c_int, [_P, _I32]),
    "adt_batch_run_resident": (C.c_int, [_P]),
    "adt_batch_download": (C.c_int, [_P, _P, _P, _P, _P]),
    "adt_batch_stream": (_P, [_P]),
    "adt_batch_device_buffer": (_P, [_P, _I32]),
    "adt_batch_stats_get": (C.c_int, [_P, _P]),
    "adt_smooth_l1": (C.c_int, [_P, _I64, _I64, _I64, _I32, _I32, _D, _P, _P]),
    "adt_smooth_l1_device": (C.c_int, [_P, _I64, _I64, _I64, _I32, _I32, _D, _P, _P, _P]),
    "adt_locate_loss_grad": (C.c_int, [_I32, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _I32, _D, _D,
                                       _D, _P, _D, _P, _P]),
}


def lib(build_if_missing: bool = True):
    """Load (building first if needed) and return the CDLL.  Raises if the
    library cannot be built or loaded -- there is no CPU fallback."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH) and build_if_missing:
                from . import build as _b
                _b.build()
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            sizes = (C.c_int64 * 3)()
            L.adt_abi_struct_sizes(sizes, 3)
            mirrors = (SolveStatus, BatchOpts, BatchStats)
            if tuple(sizes) != tuple(C.sizeof(m) for m in mirrors):
                raise AdtError(-1, f"struct sizes of {LIB_PATH} {tuple(sizes)} differ "
                                           f"from the ctypes mirrors "
                                           f"{tuple(C.sizeof(m) for m in mirrors)}")
            _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != ADT_OK:
        msg = lib().adt_last_error()
        raise AdtError(rc, msg.decode() if msg else "")
