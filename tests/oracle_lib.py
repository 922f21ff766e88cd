"""ctypes binding of the CPU oracle (oracle/nt2_oracle.c) for the tests.

The oracle is the checker: tests compare the CUDA path against it.  It is
built on first use by oracle/build_oracle.py.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_oracle  # noqa: E402

_libs = {}

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
sz = C.c_size_t

SIGS = {
    "nt2o_ulpdist_f": (C.c_double, [C.c_float, C.c_float]),
    "nt2o_ulpdist_d": (C.c_double, [C.c_double, C.c_double]),
    "nt2o_max_ulp_f": (C.c_double, [f32p, f32p, sz, C.POINTER(sz)]),
    "nt2o_max_ulp_d": (C.c_double, [f64p, f64p, sz, C.POINTER(sz)]),
    "nt2o_exp_f": (C.c_float, [C.c_float]),
    "nt2o_log_f": (C.c_float, [C.c_float]),
    "nt2o_erfc_f": (C.c_float, [C.c_float]),
    "nt2o_erfc_f_scalar": (C.c_float, [C.c_float]),
    "nt2o_normcdf_f": (C.c_float, [C.c_float]),
    "nt2o_fastnormcdf_f": (C.c_float, [C.c_float]),
    "nt2o_exp_d": (C.c_double, [C.c_double]),
    "nt2o_exp2_f": (C.c_float, [C.c_float]),
    "nt2o_expm1_f": (C.c_float, [C.c_float]),
    "nt2o_log1p_f": (C.c_float, [C.c_float]),
    "nt2o_expm1_d": (C.c_double, [C.c_double]),
    "nt2o_log1p_d": (C.c_double, [C.c_double]),
    "nt2o_sinh_f": (C.c_float, [C.c_float]),
    "nt2o_sinh_d": (C.c_double, [C.c_double]),
    "nt2o_cosh_f": (C.c_float, [C.c_float]),
    "nt2o_cosh_d": (C.c_double, [C.c_double]),
    "nt2o_tanh_f": (C.c_float, [C.c_float]),
    "nt2o_tanh_d": (C.c_double, [C.c_double]),
    "nt2o_trig_f": (C.c_int, [C.c_int, f32p, f32p, sz, C.c_int]),
    "nt2o_trig_d": (C.c_int, [C.c_int, f64p, f64p, sz, C.c_int]),
    "nt2o_atan2_f": (None, [f32p, f32p, f32p, sz]),
    "nt2o_atan2_d": (None, [f64p, f64p, f64p, sz]),
    "nt2o_pow_f": (C.c_float, [C.c_float, C.c_float]),
    "nt2o_pow_d": (C.c_double, [C.c_double, C.c_double]),
    "nt2o_pow2_f": (None, [f32p, f32p, f32p, sz]),
    "nt2o_pow2_d": (None, [f64p, f64p, f64p, sz]),
    "nt2o_trigx_f": (C.c_int, [C.c_int, f32p, f32p, sz, C.c_int]),
    "nt2o_trigx_d": (C.c_int, [C.c_int, f64p, f64p, sz, C.c_int]),
    "nt2o_map2_f": (C.c_int, [C.c_int, f32p, f32p, f32p, sz]),
    "nt2o_map2_d": (C.c_int, [C.c_int, f64p, f64p, f64p, sz]),
    "nt2o_rem_pio2_exact_f": (C.c_int, [C.c_float, C.POINTER(C.c_float)]),
    "nt2o_rem_pio2_exact_d": (C.c_int, [C.c_double, C.POINTER(C.c_double)]),
    "nt2o_exp10_f": (C.c_float, [C.c_float]),
    "nt2o_log2_f": (C.c_float, [C.c_float]),
    "nt2o_log10_f": (C.c_float, [C.c_float]),
    "nt2o_exp2_d": (C.c_double, [C.c_double]),
    "nt2o_exp10_d": (C.c_double, [C.c_double]),
    "nt2o_log2_d": (C.c_double, [C.c_double]),
    "nt2o_log10_d": (C.c_double, [C.c_double]),
    "nt2o_log_d": (C.c_double, [C.c_double]),
    "nt2o_erfc_d": (C.c_double, [C.c_double]),
    "nt2o_erfc_d_scalar": (C.c_double, [C.c_double]),
    "nt2o_normcdf_d": (C.c_double, [C.c_double]),
    "nt2o_map_f": (C.c_int, [C.c_int, f32p, f32p, sz]),
    "nt2o_map_d": (C.c_int, [C.c_int, f64p, f64p, sz]),
    "nt2o_saxpy_f": (None, [C.c_float, f32p, f32p, sz, C.c_int]),
    "nt2o_saxpy_d": (None, [C.c_double, f64p, f64p, sz, C.c_int]),
    "nt2o_rgb2grey_f": (None, [f32p, f32p, f32p, f32p, sz, C.c_int]),
    "nt2o_rgb2grey_u8": (None, [u8p, u8p, u8p, u8p, sz, C.c_int]),
    "nt2o_rgb2yuv_f": (None, [f32p, f32p, f32p, f32p, f32p, f32p, sz, C.c_int]),
    "nt2o_linspace_f": (None, [C.c_float, C.c_float, sz, f32p]),
    "nt2o_mandelbrot_f": (C.c_int, [f32p, f32p, i32p, sz, C.c_int, C.c_int]),
    "nt2o_mandelbrot_grid_f": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, sz, sz, i32p, C.c_int, C.c_int]),
    "nt2o_bs_f": (None, [f32p, f32p, f32p, C.c_float, C.c_float, f32p, f32p, sz, C.c_int, C.c_int]),
    "nt2o_bs_d": (None, [f64p, f64p, f64p, C.c_double, C.c_double, f64p, f64p, sz, C.c_int]),
    "nt2o_bs_demo_f": (None, [f32p, f32p, f32p, f32p, f32p, f32p, sz, C.c_int]),
    "nt2o_sigmadelta_u8": (None, [u8p, sz, sz, C.c_int, u8p, u8p, u8p, C.c_int, C.c_int]),
    "nt2o_sum_fp64_f": (C.c_double, [f32p, sz, C.POINTER(C.c_double)]),
    "nt2o_dot_fp64_f": (C.c_double, [f32p, f32p, sz, C.POINTER(C.c_double)]),
    "nt2o_sum_fp64_d": (C.c_double, [f64p, sz, C.POINTER(C.c_double)]),
    "nt2o_globalsum_nt2_f": (C.c_float, [f32p, sz, C.c_int]),
    "nt2o_dot_nt2_f": (C.c_float, [f32p, f32p, sz, C.c_int]),
    "nt2o_inner_fold_f": (None, [f32p, sz, sz, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "nt2o_outer_fold_f": (None, [f32p, sz, sz, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "nt2o_dot_omp_f": (C.c_float, [f32p, C.c_void_p, sz, C.c_int, C.c_int]),
    "nt2o_outer_fold_nt2_f": (None, [f32p, sz, sz, f32p, C.c_int]),
    "nt2o_sigmadelta_batch_u8": (None, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "nt2o_l2_bytes": (sz, []),
    "nt2o_max_threads": (C.c_int, []),
}

OP = {"exp": 0, "log": 1, "erfc": 2, "normcdf": 3, "fastnormcdf": 4, "sqrt": 5, "erfc_scalar": 6,
      "exp2": 7, "exp10": 8, "log2": 9, "log10": 10, "expm1": 11, "log1p": 12, "sinh": 13, "cosh": 14,
      "tanh": 15, "cbrt": 16, "sqrt1pm1": 17, "exprecneg": 18, "exprecnegc": 19, "expx2": 20,
      "realsqrt": 5, "reallog": 1, "atanh": 21, "acosh": 22, "sech": 23, "csch": 24, "acoth": 25, "asech": 26,
      "asinh": 27, "acsch": 28, "coth": 29, "sinhc": 30}
# binary functors of nt2o_map2_f/d
OP2 = {"atan2": 0, "pow": 1, "pow_abs": 2, "realpow": 3, "logspace_add": 4, "logspace_sub": 5, "expx2": 6, "atan2d": 7,
       "nbd_atan2": 8, "hypot": 9}


def load(variant: str = "libnt2oracle.so"):
    if variant in _libs:
        return _libs[variant]
    paths = build_oracle.build()
    L = C.CDLL(paths[variant])
    for name, (res, args) in SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _libs[variant] = L
    return L


def max_ulp(a: np.ndarray, b: np.ndarray):
    L = load()
    w = sz()
    if a.dtype == np.float32:
        m = L.nt2o_max_ulp_f(np.ascontiguousarray(a), np.ascontiguousarray(b), a.size, C.byref(w))
    else:
        m = L.nt2o_max_ulp_d(np.ascontiguousarray(a), np.ascontiguousarray(b), a.size, C.byref(w))
    return m, w.value


TRIG = {"sin": 0, "cos": 1, "tan": 2, "sinpi": 3, "cospi": 4, "asin": 5, "acos": 6, "atan": 7, "cot": 8, "tanpi": 9,
        "cotpi": 10, "sind": 11, "cosd": 12, "tand": 13, "cotd": 14}


def trig(op: str, x: np.ndarray, pack: int = 1) -> np.ndarray:
    """NT2's op over x in packs of `pack` lanes from index 0 and a scalar tail; pack 1 is NT2's
    scalar code, 16 // itemsize its 128-bit SIMD code."""
    L = load()
    x = np.ascontiguousarray(x)
    y = np.empty_like(x)
    fn = L.nt2o_trig_f if x.dtype == np.float32 else L.nt2o_trig_d
    assert fn(TRIG[op], x, y, x.size, pack) == 0
    return y


# trigonometric functors NT2 composes from the ones above (nt2o_trigx_f/d op numbers)
TRIGX = {"csc": 0, "sec": 1, "cscpi": 2, "secpi": 3, "cscd": 4, "indeg": 5, "inrad": 6, "acot": 7, "asind": 8,
         "acosd": 9, "atand": 10, "asinpi": 11, "acospi": 12, "atanpi": 13, "acsc": 14, "acscd": 15, "asec": 16,
         "asecd": 17, "secd": 18, "fast_sin": 19, "fast_cos": 20, "fast_tan": 21, "fast_cot": 22, "fast_sinpi": 23,
         "fast_cospi": 24, "fast_tanpi": 25, "fast_cotpi": 26, "fast_sind": 27, "fast_cosd": 28, "fast_tand": 29,
         "fast_cotd": 30, "sinc": 31, "sincpi": 32, "proper_tanpi": 33}


def trigx(op: str, x: np.ndarray, pack: int = 1) -> np.ndarray:
    """NT2's composed trigonometric functor `op`; pack as in trig()."""
    L = load()
    x = np.ascontiguousarray(x)
    y = np.empty_like(x)
    fn = L.nt2o_trigx_f if x.dtype == np.float32 else L.nt2o_trigx_d
    assert fn(TRIGX[op], x, y, x.size, pack) == 0
    return y


def atan2(a0: np.ndarray, a1: np.ndarray) -> np.ndarray:
    """NT2's atan2(a0, a1) (SIMD form), elementwise."""
    L = load()
    a0 = np.ascontiguousarray(a0)
    a1 = np.ascontiguousarray(a1, dtype=a0.dtype)
    y = np.empty_like(a0)
    (L.nt2o_atan2_f if a0.dtype == np.float32 else L.nt2o_atan2_d)(a0, a1, y, a0.size)
    return y


def pow_(a0: np.ndarray, a1: np.ndarray) -> np.ndarray:
    """NT2's pow(a0, a1) for floating a1 (SIMD form), elementwise."""
    L = load()
    a0 = np.ascontiguousarray(a0)
    a1 = np.ascontiguousarray(a1, dtype=a0.dtype)
    y = np.empty_like(a0)
    (L.nt2o_pow2_f if a0.dtype == np.float32 else L.nt2o_pow2_d)(a0, a1, y, a0.size)
    return y


def map2(op: str, a0: np.ndarray, a1: np.ndarray) -> np.ndarray:
    """NT2's binary functor `op` (SIMD form) elementwise over a0, a1."""
    L = load()
    a0 = np.ascontiguousarray(a0)
    a1 = np.ascontiguousarray(a1, dtype=a0.dtype)
    y = np.empty_like(a0)
    fn = L.nt2o_map2_f if a0.dtype == np.float32 else L.nt2o_map2_d
    assert fn(OP2[op], a0, a1, y, a0.size) == 0
    return y


def map_(op: str, x: np.ndarray) -> np.ndarray:
    if op in TRIG:
        return trig(op, x)
    if op in TRIGX:
        return trigx(op, x)
    L = load()
    y = np.empty_like(x)
    fn = L.nt2o_map_f if x.dtype == np.float32 else L.nt2o_map_d
    assert fn(OP[op], x, y, x.size) == 0
    return y


def bs(S, K, T, r, v, cdf: int = 0, threads: int = 0):
    L = load()
    call = np.empty_like(S)
    put = np.empty_like(S)
    if S.dtype == np.float32:
        L.nt2o_bs_f(S, K, T, r, v, call, put, S.size, cdf, threads)
    else:
        L.nt2o_bs_d(S, K, T, r, v, call, put, S.size, threads)
    return call, put


def bs_demo(S, X, T, r, v, threads: int = 0):
    R = np.empty_like(S)
    load().nt2o_bs_demo_f(S, X, T, r, v, R, S.size, threads)
    return R


def sigmadelta(frames: np.ndarray, frame_stride: int, npix: int, nframes: int, bkg=None, var=None,
               init: bool = True, threads: int = 0):
    bkg = np.zeros(npix, np.uint8) if bkg is None else bkg.copy()
    var = np.zeros(npix, np.uint8) if var is None else var.copy()
    nl = nframes - 1 if init else nframes
    labels = np.zeros(max(nl, 1) * npix, np.uint8)
    load().nt2o_sigmadelta_u8(frames, frame_stride, npix, nframes, bkg, var, labels, int(init), threads)
    return bkg, var, labels[: nl * npix]


def inner_fold(A, rows, cols, lanes=8):
    out32 = np.empty(cols, np.float32)
    out64 = np.empty(cols, np.float64)
    abs64 = np.empty(cols, np.float64)
    load().nt2o_inner_fold_f(A, rows, cols, lanes, out32.ctypes.data, out64.ctypes.data, abs64.ctypes.data, 0)
    return out32, out64, abs64


def outer_fold(A, rows, cols):
    out32 = np.empty(rows, np.float32)
    out64 = np.empty(rows, np.float64)
    abs64 = np.empty(rows, np.float64)
    load().nt2o_outer_fold_f(A, rows, cols, out32.ctypes.data, out64.ctypes.data, abs64.ctypes.data, 0)
    return out32, out64, abs64


def sum_fp64(x):
    a = C.c_double()
    if x.dtype == np.float32:
        s = load().nt2o_sum_fp64_f(x, x.size, C.byref(a))
    else:
        s = load().nt2o_sum_fp64_d(x, x.size, C.byref(a))
    return s, a.value


def dot_fp64(x, y):
    a = C.c_double()
    s = load().nt2o_dot_fp64_f(x, y, x.size, C.byref(a))
    return s, a.value


def rgb2yuv(r, g, b, threads: int = 0):
    y, u, v = (np.empty_like(r) for _ in range(3))
    load().nt2o_rgb2yuv_f(r, g, b, y, u, v, r.size, threads)
    return y, u, v


def mandelbrot(A, B, pack: int = 8, threads: int = 0):
    C_ = np.empty(A.size, np.int32)
    assert load().nt2o_mandelbrot_f(np.ascontiguousarray(A), np.ascontiguousarray(B), C_, A.size, pack, threads) == 0
    return C_


def mandelbrot_grid(a0, a1, b0, b1, h, w, pack: int = 8, threads: int = 0):
    C_ = np.empty(h * w, np.int32)
    assert load().nt2o_mandelbrot_grid_f(a0, a1, b0, b1, h, w, C_, pack, threads) == 0
    return C_


def linspace(lo, hi, n):
    out = np.empty(max(n, 1), np.float32)
    load().nt2o_linspace_f(lo, hi, n, out)
    return out[:n]
