"""ctypes binding of libnt2cuda.so (the C ABI declared in include/nt2cuda.h).

The library is built in-tree by nt2_gb300.build.  Loading fails loudly when
it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnt2cuda.so")

_lock = threading.Lock()
_lib = None

c_size = C.c_size_t
c_vp = C.c_void_p
c_int = C.c_int
c_f = C.c_float
c_d = C.c_double
c_u64 = C.c_uint64


class NT2CudaError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = _lib.nt2cuda_status_string(status).decode() if _lib else str(status)
        super().__init__(f"{where}: nt2cuda status {status} ({msg})")


class SdStream(C.Structure):
    """nt2cuda_sd_stream."""
    _fields_ = [
        ("frames", c_vp), ("frame_stride", c_size), ("bkg", c_vp), ("var", c_vp),
        ("labels", c_vp), ("label_stride", c_size), ("width", C.c_uint32), ("height", C.c_uint32),
    ]


class ServerConfig(C.Structure):
    """nt2cuda_server_config."""
    _fields_ = [
        ("budget_bytes", c_size), ("max_batch_requests", c_int), ("max_inflight_batches", c_int),
        ("coalesce", c_int), ("fused", c_int), ("cdf_kind", c_int), ("wait_timeout_ms", c_int),
        ("spin_us", c_int),
    ]


class ServerStats(C.Structure):
    """nt2cuda_server_stats."""
    _fields_ = [
        ("submitted", c_u64), ("completed", c_u64), ("batches", c_u64), ("launches", c_u64),
        ("options", c_u64), ("reserved_bytes", c_size), ("peak_reserved_bytes", c_size),
        ("admission_waits", c_u64),
    ]


# name -> (restype, argtypes)
_SIGS = {
    "nt2cuda_status_string": (C.c_char_p, [c_int]),
    "nt2cuda_version": (c_int, []),
    "nt2cuda_init": (c_int, [c_int]),
    "nt2cuda_device_info": (c_int, [C.POINTER(c_int), C.POINTER(c_size), C.POINTER(c_size)]),
    "nt2cuda_last_cuda_error": (c_int, [C.POINTER(c_int)]),
    "nt2cuda_scratch_allocations": (c_int, [C.POINTER(C.c_ulonglong)]),
    "nt2cuda_alloc": (c_int, [c_size, C.POINTER(c_vp)]),
    "nt2cuda_free": (c_int, [c_vp]),
    "nt2cuda_alloc_host": (c_int, [c_size, C.POINTER(c_vp)]),
    "nt2cuda_free_host": (c_int, [c_vp]),
    "nt2cuda_memcpy_h2d": (c_int, [c_vp, c_vp, c_size, c_vp]),
    "nt2cuda_memcpy_d2h": (c_int, [c_vp, c_vp, c_size, c_vp]),
    "nt2cuda_memcpy_d2d": (c_int, [c_vp, c_vp, c_size, c_vp]),
    "nt2cuda_stream_create": (c_int, [C.POINTER(c_vp)]),
    "nt2cuda_stream_destroy": (c_int, [c_vp]),
    "nt2cuda_stream_sync": (c_int, [c_vp]),
    "nt2cuda_map_f32": (c_int, [c_int, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_map_f64": (c_int, [c_int, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_saxpy_f32": (c_int, [c_f, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_saxpy_f64": (c_int, [c_d, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_rgb2grey_f32": (c_int, [c_vp, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_reduce_f32": (c_int, [c_int, c_vp, c_size, c_size, c_int, c_vp, c_int, c_vp]),
    "nt2cuda_reduce_f64": (c_int, [c_int, c_vp, c_size, c_size, c_int, c_vp, c_int, c_vp]),
    "nt2cuda_reduce_logical_f32": (c_int, [c_int, c_vp, c_size, c_size, c_int, c_vp, c_vp]),
    "nt2cuda_reduce_logical_f64": (c_int, [c_int, c_vp, c_size, c_size, c_int, c_vp, c_vp]),
    "nt2cuda_scan_f32": (c_int, [c_int, c_vp, c_size, c_size, c_int, c_vp, c_int, c_vp]),
    "nt2cuda_wait_timeouts": (c_int, [C.POINTER(C.c_ulonglong)]),
    "nt2cuda_atan2_f32": (c_int, [c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_atan2_f64": (c_int, [c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_pow_f32": (c_int, [c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_pow_f64": (c_int, [c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_sincos_f32": (c_int, [c_int, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_sincos_f64": (c_int, [c_int, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_map2_f32": (c_int, [c_int, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_map2_f64": (c_int, [c_int, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_selftest_wait_timeout": (c_int, [c_vp]),
    "nt2cuda_selftest_fold_timeout": (c_int, [c_vp, c_size, c_size, c_vp, c_vp]),
    "nt2cuda_selftest_x2": (c_int, [c_int, C.POINTER(C.c_ulonglong), C.POINTER(C.c_uint32), c_vp]),
    "nt2cuda_scan_f64": (c_int, [c_int, c_vp, c_size, c_size, c_int, c_vp, c_int, c_vp]),
    "nt2cuda_rgb2grey_u8": (c_int, [c_vp, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_rgb2yuv_f32": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_mandelbrot_f32": (c_int, [c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_mandelbrot_grid_f32": (c_int, [c_f, c_f, c_f, c_f, c_size, c_size, c_vp, c_int, c_vp]),
    "nt2cuda_blackscholes_f32": (c_int, [c_vp, c_vp, c_vp, c_f, c_f, c_vp, c_vp, c_size, c_int, c_int, c_vp]),
    "nt2cuda_blackscholes_f64": (c_int, [c_vp, c_vp, c_vp, c_d, c_d, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_blackscholes_demo_f32": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_size, c_int, c_vp]),
    "nt2cuda_blackscholes_f32_host": (c_int, [c_vp, c_vp, c_vp, c_f, c_f, c_vp, c_vp, c_size, c_int, c_int]),
    "nt2cuda_globalsum_f32": (c_int, [c_vp, c_size, c_vp, c_int, c_vp]),
    "nt2cuda_dot_f32": (c_int, [c_vp, c_vp, c_size, c_vp, c_int, c_vp]),
    "nt2cuda_dot_f32_noalloc": (c_int, [c_vp, c_vp, c_size, c_vp, c_int, c_vp]),
    "nt2cuda_globalsum_f64": (c_int, [c_vp, c_size, c_vp, c_vp]),
    "nt2cuda_dot_f64": (c_int, [c_vp, c_vp, c_size, c_vp, c_vp]),
    "nt2cuda_sum_inner_f32": (c_int, [c_vp, c_size, c_size, c_vp, c_int, c_vp]),
    "nt2cuda_sum_inner_f64": (c_int, [c_vp, c_size, c_size, c_vp, c_vp]),
    "nt2cuda_sum_outer_f32": (c_int, [c_vp, c_size, c_size, c_vp, c_int, c_vp]),
    "nt2cuda_sum_outer_f64": (c_int, [c_vp, c_size, c_size, c_vp, c_vp]),
    "nt2cuda_set_fold_path": (c_int, [c_int]),
    "nt2cuda_sigmadelta_batch_u8": (c_int, [C.POINTER(SdStream), c_int, c_int, c_int, c_vp]),
    "nt2cuda_sigmadelta_plan_create": (c_int, [C.POINTER(SdStream), c_int, c_int, c_int, c_vp, C.POINTER(c_vp)]),
    "nt2cuda_sigmadelta_plan_launch": (c_int, [c_vp, c_vp]),
    "nt2cuda_sigmadelta_plan_destroy": (c_int, [c_vp]),
    "nt2cuda_autotune": (c_int, [C.c_char_p, c_size, C.POINTER(c_int), C.POINTER(c_int), C.POINTER(c_f)]),
    "nt2cuda_tuning_export": (c_int, [C.c_char_p, c_size, C.POINTER(c_size)]),
    "nt2cuda_tuning_import": (c_int, [C.c_char_p, C.POINTER(c_int)]),
    "nt2cuda_fill_uniform_f32": (c_int, [c_vp, c_size, c_f, c_f, c_u64, c_vp]),
    "nt2cuda_fill_uniform_f64": (c_int, [c_vp, c_size, c_d, c_d, c_u64, c_vp]),
    "nt2cuda_fill_normal_f32": (c_int, [c_vp, c_size, c_u64, c_vp]),
    "nt2cuda_server_create": (c_int, [C.POINTER(ServerConfig), C.POINTER(c_vp)]),
    "nt2cuda_server_destroy": (c_int, [c_vp]),
    "nt2cuda_server_submit": (c_int, [c_vp, c_vp, c_vp, c_vp, c_f, c_f, c_size, C.POINTER(c_u64)]),
    "nt2cuda_server_poll": (c_int, [c_vp, c_u64, C.POINTER(c_vp), C.POINTER(c_vp)]),
    "nt2cuda_server_wait": (c_int, [c_vp, c_u64, c_int, C.POINTER(c_vp), C.POINTER(c_vp)]),
    "nt2cuda_server_release": (c_int, [c_vp, c_u64]),
    "nt2cuda_server_latency_ns": (c_int, [c_vp, c_u64, C.POINTER(c_u64)]),
    "nt2cuda_server_drain": (c_int, [c_vp, c_int]),
    "nt2cuda_server_get_stats": (c_int, [c_vp, C.POINTER(ServerStats)]),
    "nt2cuda_server_replay": (c_int, [c_vp, c_vp, c_vp, c_vp, c_f, c_f, c_size, c_vp, c_vp, c_vp, c_vp, c_vp]),
}


def lib():
    """Load (once) and return the ctypes handle.  Raises if the library is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"nt2cuda extension not built ({LIB_PATH} missing); "
                "run `python -c 'import nt2_gb300.build as b; b.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str = "nt2cuda") -> None:
    if status != 0:
        raise NT2CudaError(status, where)


def declared_symbols() -> list[str]:
    return sorted(_SIGS)
