"""Table-expression evaluation on the GPU through the nt2cuda C ABI.

Functions take torch tensors as tables (device memory owned by torch) and
call the C entry points on torch's current CUDA stream, so they compose
with torch work.  Names and argument meanings follow NT2's
(saxpy, blackscholes, globalsum, sum(A, dim), sigmadelta).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import torch

from ._lib import SdStream, check, lib

OPS = {"exp": 0, "log": 1, "erfc": 2, "normcdf": 3, "fastnormcdf": 4, "sqrt": 5, "exp2": 6, "exp10": 7, "log2": 8,
       "log10": 9, "expm1": 10, "log1p": 11, "sin": 12, "cos": 13, "tan": 14, "sinpi": 15, "cospi": 16,
       "asin": 17, "acos": 18, "atan": 19, "sinh": 20, "cosh": 21, "tanh": 22, "cbrt": 23, "sqrt1pm1": 24,
       "exprecneg": 25, "exprecnegc": 26, "expx2": 27, "realsqrt": 28, "reallog": 29, "csc": 30, "sec": 31,
       "cscpi": 32, "secpi": 33, "cscd": 34, "indeg": 35, "inrad": 36, "acot": 37, "asind": 38, "acosd": 39,
       "atand": 40, "asinpi": 41, "acospi": 42, "atanpi": 43, "acsc": 44, "acscd": 45, "asec": 46, "asecd": 47,
       "cot": 48, "tanpi": 49, "cotpi": 50, "sind": 51, "cosd": 52, "tand": 53, "cotd": 54, "secd": 55,
       "fast_sin": 56, "fast_cos": 57, "fast_tan": 58, "fast_cot": 59, "fast_sinpi": 60, "fast_cospi": 61,
       "fast_tanpi": 62, "fast_cotpi": 63, "fast_sind": 64, "fast_cosd": 65, "fast_tand": 66, "fast_cotd": 67,
       "sinc": 68, "sincpi": 69, "atanh": 70, "acosh": 71, "sech": 72, "csch": 73, "acoth": 74, "asech": 75, "asinh": 76, "acsch": 77, "coth": 78, "sinhc": 79, "proper_tanpi": 80}
# binary functors of nt2cuda_map2_f32/f64
OPS2 = {"atan2": 0, "pow": 1, "pow_abs": 2, "realpow": 3, "logspace_add": 4, "logspace_sub": 5, "expx2": 6,
        "atan2d": 7, "nbd_atan2": 8, "hypot": 9}
CDF = {"normcdf": 0, "fastnormcdf": 1}


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _dev(t: torch.Tensor, dtype=None, name: str = "table") -> int:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    return t.data_ptr()


def init(device: int = 0) -> None:
    check(lib().nt2cuda_init(device), "init")


MAP_FUSED, MAP_SIMD128 = 1, 2


def map_(op: str, x: torch.Tensor, out: torch.Tensor | None = None, fused: bool = False,
         simd128: bool = False) -> torch.Tensor:
    """out = nt2::op(x) for op in exp, log, erfc, normcdf, fastnormcdf, sqrt, exp2, exp10, log2, log10, expm1,
    log1p, sin, cos, tan, sinpi, cospi, asin, acos, atan, sinh, cosh, tanh, cbrt, sqrt1pm1, exprecneg, exprecnegc,
    expx2, realsqrt, reallog and the composed trigonometric ops (csc, sec, cscpi, secpi, cscd, indeg, inrad,
    acot, asind, acosd, atand, asinpi, acospi, atanpi, acsc, acscd, asec, asecd), cot, tanpi, cotpi and the degree
    forms sind, cosd, tand, cotd, secd, the fast_ forms (fast_sin ... fast_cotd), sinc, sincpi, and atanh, acosh,
    sech, csch, acoth, asech, asinh, acsch, coth, sinhc, proper_tanpi.  The
    trigonometric ops reduce each
    element on its own (NT2's scalar
    code); with simd128 they reduce each 16-byte pack of x with the method NT2's 128-bit SIMD code picks for
    the pack's largest |x| (tables that are not 16-byte aligned: scalar code throughout)."""
    out = torch.empty_like(x) if out is None else out
    L = lib()
    flags = (MAP_FUSED if fused else 0) | (MAP_SIMD128 if simd128 else 0)
    if x.dtype == torch.float32:
        st = L.nt2cuda_map_f32(OPS[op], _dev(x), _dev(out, torch.float32), x.numel(), flags, _stream())
    elif x.dtype == torch.float64:
        st = L.nt2cuda_map_f64(OPS[op], _dev(x), _dev(out, torch.float64), x.numel(), flags, _stream())
    else:
        raise TypeError("map_ takes float32 or float64 tables")
    check(st, f"map_({op})")
    return out


def _binary(name: str, a0: torch.Tensor, a1: torch.Tensor, out: torch.Tensor | None, fused: bool) -> torch.Tensor:
    if a0.numel() != a1.numel():
        raise ValueError("a0 and a1 must have the same size")
    out = torch.empty_like(a0) if out is None else out
    L = lib()
    if a0.dtype == torch.float32:
        st = getattr(L, f"nt2cuda_{name}_f32")(_dev(a0), _dev(a1, torch.float32), _dev(out, torch.float32),
                                               a0.numel(), MAP_FUSED if fused else 0, _stream())
    elif a0.dtype == torch.float64:
        st = getattr(L, f"nt2cuda_{name}_f64")(_dev(a0), _dev(a1, torch.float64), _dev(out, torch.float64),
                                               a0.numel(), MAP_FUSED if fused else 0, _stream())
    else:
        raise TypeError(f"{name} takes float32 or float64 tables")
    check(st, name)
    return out


def map2(op: str, a0: torch.Tensor, a1: torch.Tensor, out: torch.Tensor | None = None,
         fused: bool = False) -> torch.Tensor:
    """out = nt2::op(a0, a1) elementwise over two tables of one floating type, op in OPS2."""
    if a0.numel() != a1.numel():
        raise ValueError("a0 and a1 must have the same size")
    out = torch.empty_like(a0) if out is None else out
    L = lib()
    if a0.dtype == torch.float32:
        st = L.nt2cuda_map2_f32(OPS2[op], _dev(a0), _dev(a1, torch.float32), _dev(out, torch.float32),
                                a0.numel(), MAP_FUSED if fused else 0, _stream())
    elif a0.dtype == torch.float64:
        st = L.nt2cuda_map2_f64(OPS2[op], _dev(a0), _dev(a1, torch.float64), _dev(out, torch.float64),
                                a0.numel(), MAP_FUSED if fused else 0, _stream())
    else:
        raise TypeError(f"{op} takes float32 or float64 tables")
    check(st, f"map2({op})")
    return out


SINCOS = {"sincos": 0, "sincospi": 1, "sincosd": 2, "fast_sincos": 3, "fast_sincospi": 4, "fast_sincosd": 5,
          "sinhcosh": 6}


def sincos(x: torch.Tensor, form: str = "sincos", s: torch.Tensor | None = None, c: torch.Tensor | None = None,
           fused: bool = False, simd128: bool = False) -> tuple[torch.Tensor, torch.Tensor]:
    """tie(s, c) = nt2::sincos(x) (or sincospi, sincosd, fast_sincos, fast_sincospi, fast_sincosd, sinhcosh) in one
    pass."""
    s = torch.empty_like(x) if s is None else s
    c = torch.empty_like(x) if c is None else c
    flags = (MAP_FUSED if fused else 0) | (MAP_SIMD128 if simd128 else 0)
    L = lib()
    if x.dtype == torch.float32:
        st = L.nt2cuda_sincos_f32(SINCOS[form], _dev(x), _dev(s, torch.float32), _dev(c, torch.float32), x.numel(),
                                  flags, _stream())
    elif x.dtype == torch.float64:
        st = L.nt2cuda_sincos_f64(SINCOS[form], _dev(x), _dev(s, torch.float64), _dev(c, torch.float64), x.numel(),
                                  flags, _stream())
    else:
        raise TypeError("sincos takes float32 or float64 tables")
    check(st, form)
    return s, c


def atan2(a0: torch.Tensor, a1: torch.Tensor, out: torch.Tensor | None = None, fused: bool = False) -> torch.Tensor:
    """out = nt2::atan2(a0, a1) elementwise (NT2's SIMD form)."""
    return _binary("atan2", a0, a1, out, fused)


def pow(a0: torch.Tensor, a1: torch.Tensor, out: torch.Tensor | None = None, fused: bool = False) -> torch.Tensor:
    """out = nt2::pow(a0, a1) elementwise for a floating exponent table (NT2's SIMD form)."""
    return _binary("pow", a0, a1, out, fused)


def saxpy(alpha: float, x: torch.Tensor, y: torch.Tensor, fused: bool = False) -> torch.Tensor:
    """Y = alpha*X + Y, in place."""
    if x.numel() != y.numel():
        raise ValueError("x and y must have the same size")
    L = lib()
    if y.dtype == torch.float32:
        st = L.nt2cuda_saxpy_f32(alpha, _dev(x, torch.float32), _dev(y), y.numel(), int(fused), _stream())
    elif y.dtype == torch.float64:
        st = L.nt2cuda_saxpy_f64(alpha, _dev(x, torch.float64), _dev(y), y.numel(), int(fused), _stream())
    else:
        raise TypeError("saxpy takes float32 or float64 tables")
    check(st, "saxpy")
    return y


def rgb2grey(r: torch.Tensor, g: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None,
             fused: bool = False) -> torch.Tensor:
    """gr = 0.3*r + 0.59*g + 0.11*b over float32 planes, or over uint8 planes with the
    float statement between cast<float> and cast<uint8_t>."""
    out = torch.empty_like(r) if out is None else out
    if r.dtype == torch.uint8:
        st = lib().nt2cuda_rgb2grey_u8(_dev(r, torch.uint8), _dev(g, torch.uint8), _dev(b, torch.uint8),
                                       _dev(out, torch.uint8), r.numel(), int(fused), _stream())
    else:
        st = lib().nt2cuda_rgb2grey_f32(_dev(r, torch.float32), _dev(g, torch.float32), _dev(b, torch.float32),
                                        _dev(out, torch.float32), r.numel(), int(fused), _stream())
    check(st, "rgb2grey")
    return out


def rgb2yuv(r: torch.Tensor, g: torch.Tensor, b: torch.Tensor, fused: bool = False):
    """(y, u, v) of the rgb2yuv demo over float32 planes, in one pass."""
    y, u, v = (torch.empty_like(r) for _ in range(3))
    check(lib().nt2cuda_rgb2yuv_f32(_dev(r, torch.float32), _dev(g, torch.float32), _dev(b, torch.float32),
                                    _dev(y), _dev(u), _dev(v), r.numel(), int(fused), _stream()), "rgb2yuv")
    return y, u, v


def mandelbrot(A: torch.Tensor, B: torch.Tensor, pack: int = 8, out: torch.Tensor | None = None) -> torch.Tensor:
    """C = arrayfun(step, A, B) of the mandelbrot demo: int32 escape counts (at most 256)."""
    if A.numel() != B.numel():
        raise ValueError("A and B must have the same size")
    out = torch.empty(A.shape, dtype=torch.int32, device=A.device) if out is None else out
    check(lib().nt2cuda_mandelbrot_f32(_dev(A, torch.float32), _dev(B, torch.float32), _dev(out, torch.int32),
                                       A.numel(), int(pack), _stream()), "mandelbrot")
    return out


def mandelbrot_grid(a0: float, a1: float, b0: float, b1: float, h: int, w: int, pack: int = 8,
                    out: torch.Tensor | None = None) -> torch.Tensor:
    """The demo's whole program over an h x w grid (column-major, returned as a flat int32 table)."""
    out = torch.empty(h * w, dtype=torch.int32, device="cuda") if out is None else out
    if out.numel() != h * w:
        raise ValueError("out must hold h*w counts")
    check(lib().nt2cuda_mandelbrot_grid_f32(a0, a1, b0, b1, h, w, _dev(out, torch.int32), int(pack), _stream()),
          "mandelbrot_grid")
    return out


PRECISION = {"exact": 0, "fused": 1, "fast": 2}


def _prec(fused, precision):
    if precision is not None:
        return PRECISION[precision]
    return 1 if fused else 0


def blackscholes(S: torch.Tensor, K: torch.Tensor, T: torch.Tensor, r: float, sigma: float,
                 call: torch.Tensor | None = None, put: torch.Tensor | None = None,
                 cdf: str = "normcdf", fused: bool = False, precision: str | None = None):
    """(call, put) prices for n options; float32 or float64 tables.

    precision: "exact" (bit-exact NT2 arithmetic, default), "fused" (hardware FMA) or "fast"."""
    n = S.numel()
    if K.numel() != n or T.numel() != n:
        raise ValueError("S, K, T must have the same size")
    call = torch.empty_like(S) if call is None else call
    put = torch.empty_like(S) if put is None else put
    L = lib()
    if S.dtype == torch.float32:
        st = L.nt2cuda_blackscholes_f32(_dev(S), _dev(K, torch.float32), _dev(T, torch.float32), r, sigma,
                                        _dev(call, torch.float32), _dev(put, torch.float32), n, CDF[cdf],
                                        _prec(fused, precision), _stream())
    elif S.dtype == torch.float64:
        if cdf != "normcdf":
            raise ValueError("fastnormcdf is float32 only")
        st = L.nt2cuda_blackscholes_f64(_dev(S), _dev(K, torch.float64), _dev(T, torch.float64), r, sigma,
                                        _dev(call, torch.float64), _dev(put, torch.float64), n,
                                        _prec(fused, precision), _stream())
    else:
        raise TypeError("blackscholes takes float32 or float64 tables")
    check(st, "blackscholes")
    return call, put


def blackscholes_demo(S, X, T, r, v, out=None, fused: bool = False) -> torch.Tensor:
    """The demo statement with five float32 tables (r and v are tables)."""
    out = torch.empty_like(S) if out is None else out
    check(lib().nt2cuda_blackscholes_demo_f32(_dev(S, torch.float32), _dev(X, torch.float32),
                                              _dev(T, torch.float32), _dev(r, torch.float32),
                                              _dev(v, torch.float32), _dev(out, torch.float32), S.numel(),
                                              int(fused), _stream()), "blackscholes_demo")
    return out


def blackscholes_host(S, K, T, r: float, sigma: float, call, put, cdf: str = "normcdf", fused: bool = False,
                      precision: str | None = None):
    """Host-buffer form: S, K, T, call, put are CPU float32 tensors (pinned for best speed)."""
    for t in (S, K, T, call, put):
        if t.is_cuda or not t.is_contiguous() or t.dtype != torch.float32:
            raise ValueError("host tables must be contiguous CPU float32 tensors")
    check(lib().nt2cuda_blackscholes_f32_host(S.data_ptr(), K.data_ptr(), T.data_ptr(), r, sigma, call.data_ptr(),
                                              put.data_ptr(), S.numel(), CDF[cdf], _prec(fused, precision)),
          "blackscholes_host")
    return call, put


def globalsum(x: torch.Tensor, compensated: bool = True, out: torch.Tensor | None = None) -> torch.Tensor:
    """globalsum(X) as a 1-element device table."""
    out = torch.empty(1, dtype=x.dtype, device=x.device) if out is None else out
    L = lib()
    if x.dtype == torch.float32:
        st = L.nt2cuda_globalsum_f32(_dev(x), x.numel(), _dev(out, torch.float32), int(compensated), _stream())
    elif x.dtype == torch.float64:
        st = L.nt2cuda_globalsum_f64(_dev(x), x.numel(), _dev(out, torch.float64), _stream())
    else:
        raise TypeError("globalsum takes float32 or float64 tables")
    check(st, "globalsum")
    return out


def dot(x: torch.Tensor, y: torch.Tensor, compensated: bool = True, out: torch.Tensor | None = None):
    """globalsum(X*Y) (the sdot demo) as a 1-element device table."""
    if x.numel() != y.numel():
        raise ValueError("x and y must have the same size")
    out = torch.empty(1, dtype=x.dtype, device=x.device) if out is None else out
    L = lib()
    if x.dtype == torch.float32:
        st = L.nt2cuda_dot_f32(_dev(x), _dev(y, torch.float32), x.numel(), _dev(out, torch.float32),
                               int(compensated), _stream())
    elif x.dtype == torch.float64:
        st = L.nt2cuda_dot_f64(_dev(x), _dev(y, torch.float64), x.numel(), _dev(out, torch.float64), _stream())
    else:
        raise TypeError("dot takes float32 or float64 tables")
    check(st, "dot")
    return out


def sum_colmajor(A: torch.Tensor, rows: int, cols: int, dim: int, compensated: bool = True,
                 out: torch.Tensor | None = None) -> torch.Tensor:
    """sum(A, dim) of a rows x cols column-major table stored flat in A (NT2 layout).

    dim = 1: column sums (inner_fold) -> cols values; dim = 2: row sums (outer_fold) -> rows values.
    """
    if A.numel() != rows * cols:
        raise ValueError("A must hold rows*cols elements")
    if dim not in (1, 2):
        raise ValueError("dim must be 1 or 2")
    m = cols if dim == 1 else rows
    out = torch.empty(m, dtype=A.dtype, device=A.device) if out is None else out
    L = lib()
    if A.dtype == torch.float32:
        fn = L.nt2cuda_sum_inner_f32 if dim == 1 else L.nt2cuda_sum_outer_f32
        st = fn(_dev(A), rows, cols, _dev(out, torch.float32), int(compensated), _stream())
    elif A.dtype == torch.float64:
        fn = L.nt2cuda_sum_inner_f64 if dim == 1 else L.nt2cuda_sum_outer_f64
        st = fn(_dev(A), rows, cols, _dev(out, torch.float64), _stream())
    else:
        raise TypeError("sum takes float32 or float64 tables")
    check(st, f"sum(A,{dim})")
    return out


REDUCTIONS = {"sum": 0, "asum1": 1, "asum2": 2, "norm2": 3, "mean": 4, "var": 5, "stdev": 6, "max": 7, "min": 8,
              "prod": 9}
LOGICAL_REDUCTIONS = {"all": 0, "any": 1, "none": 2}


def reduce(op: str, A: torch.Tensor, rows: int, cols: int, dim: int = 1, compensated: bool = True,
           var_by_n: bool = False, out: torch.Tensor | None = None) -> torch.Tensor:
    """NT2's reductions of a rows x cols column-major table stored flat in A.

    op: sum, asum1, asum2, norm2, mean, var, stdev, max, min, prod (values of A's type) or
    all, any, none (uint8 0/1).  dim = 1: one value per column; 2: one per row; 0: the whole
    table (NT2's global* functions).  var_by_n: NT2's w = 1 (normalise by n instead of n - 1).
    """
    if A.numel() != rows * cols:
        raise ValueError("A must hold rows*cols elements")
    if dim not in (0, 1, 2):
        raise ValueError("dim must be 0, 1 or 2")
    m = 1 if dim == 0 else (cols if dim == 1 else rows)
    L = lib()
    if A.dtype not in (torch.float32, torch.float64):
        raise TypeError("reductions take float32 or float64 tables")
    f32 = A.dtype == torch.float32
    if op in LOGICAL_REDUCTIONS:
        out = torch.empty(m, dtype=torch.uint8, device=A.device) if out is None else out
        fn = L.nt2cuda_reduce_logical_f32 if f32 else L.nt2cuda_reduce_logical_f64
        st = fn(LOGICAL_REDUCTIONS[op], _dev(A), rows, cols, dim, _dev(out, torch.uint8), _stream())
    else:
        out = torch.empty(m, dtype=A.dtype, device=A.device) if out is None else out
        flags = (0 if compensated else 1) | (2 if var_by_n else 0)
        fn = L.nt2cuda_reduce_f32 if f32 else L.nt2cuda_reduce_f64
        st = fn(REDUCTIONS[op], _dev(A), rows, cols, dim, _dev(out, A.dtype), flags, _stream())
    check(st, f"{op}(A,{dim})")
    return out


SCANS = {"cumsum": 0, "cumprod": 1, "cummax": 2, "cummin": 3}


def cumulative(op: str, A: torch.Tensor, rows: int, cols: int, dim: int = 1, compensated: bool = True,
               out: torch.Tensor | None = None) -> torch.Tensor:
    """cumsum / cumprod / cummax / cummin of a rows x cols column-major table stored flat in A,
    down each column (dim 1) or along each row (dim 2); out may be A (in place)."""
    if A.numel() != rows * cols:
        raise ValueError("A must hold rows*cols elements")
    if dim not in (1, 2):
        raise ValueError("dim must be 1 or 2")
    out = torch.empty_like(A) if out is None else out
    L = lib()
    if A.dtype == torch.float32:
        fn = L.nt2cuda_scan_f32
    elif A.dtype == torch.float64:
        fn = L.nt2cuda_scan_f64
    else:
        raise TypeError("cumulative functions take float32 or float64 tables")
    check(fn(SCANS[op], _dev(A), rows, cols, dim, _dev(out, A.dtype), 0 if compensated else 1, _stream()),
          f"{op}(A,{dim})")
    return out


def sd_streams(entries: Sequence[dict]) -> C.Array:
    """Build an nt2cuda_sd_stream array from dicts of tensors and sizes."""
    arr = (SdStream * len(entries))()
    for i, e in enumerate(entries):
        arr[i] = SdStream(_dev(e["frames"], torch.uint8), e["frame_stride"], _dev(e["bkg"], torch.uint8),
                          _dev(e["var"], torch.uint8), _dev(e["labels"], torch.uint8), e["label_stride"],
                          e["width"], e["height"])
    return arr


def sigmadelta_batch(entries: Sequence[dict], nframes: int, init: bool = True) -> None:
    arr = sd_streams(entries)
    check(lib().nt2cuda_sigmadelta_batch_u8(arr, len(entries), nframes, int(init), _stream()), "sigmadelta_batch")


class SigmaDeltaPlan:
    """The batched sigma-delta launch captured once in a CUDA graph."""

    def __init__(self, entries: Sequence[dict], nframes: int, init: bool = True):
        self._arr = sd_streams(entries)
        self._p = C.c_void_p()
        check(lib().nt2cuda_sigmadelta_plan_create(self._arr, len(entries), nframes, int(init), _stream(),
                                                   C.byref(self._p)), "sigmadelta_plan_create")

    def launch(self) -> None:
        check(lib().nt2cuda_sigmadelta_plan_launch(self._p, _stream()), "sigmadelta_plan_launch")

    def close(self) -> None:
        if self._p:
            lib().nt2cuda_sigmadelta_plan_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fill_uniform(x: torch.Tensor, lo: float, hi: float, seed: int) -> torch.Tensor:
    L = lib()
    if x.dtype == torch.float32:
        st = L.nt2cuda_fill_uniform_f32(_dev(x), x.numel(), lo, hi, seed, _stream())
    elif x.dtype == torch.float64:
        st = L.nt2cuda_fill_uniform_f64(_dev(x), x.numel(), lo, hi, seed, _stream())
    else:
        raise TypeError("fill_uniform takes float32 or float64 tables")
    check(st, "fill_uniform")
    return x


def fill_normal(x: torch.Tensor, seed: int) -> torch.Tensor:
    check(lib().nt2cuda_fill_normal_f32(_dev(x, torch.float32), x.numel(), seed, _stream()), "fill_normal")
    return x


def autotune(kernel: str, n: int):
    u, w, ms = C.c_int(), C.c_int(), C.c_float()
    check(lib().nt2cuda_autotune(kernel.encode(), n, C.byref(u), C.byref(w), C.byref(ms)), "autotune")
    return u.value, w.value, ms.value


def tuning_export() -> str:
    L = lib()
    need = C.c_size_t()
    check(L.nt2cuda_tuning_export(None, 0, C.byref(need)), "tuning_export")
    buf = C.create_string_buffer(need.value)
    check(L.nt2cuda_tuning_export(buf, need.value, C.byref(need)), "tuning_export")
    return buf.value.decode()


def tuning_import(text: str) -> int:
    n = C.c_int()
    check(lib().nt2cuda_tuning_import(text.encode(), C.byref(n)), "tuning_import")
    return n.value
