// trigx_impl.cuh -- the trigonometric functors NT2 composes from sin, cos,
// sinpi, cospi, asin, acos, atan, and cot with the pi- and degree-unit
// functors (ops NT2CUDA_OP_CSC..NT2CUDA_OP_SECD of
// nt2cuda_map_f32/f64), lowered as expression trees onto the elementwise
// transform: csc(x) is rec(sin(x)) evaluated in one pass, the sine part in
// the scalar or the 128-bit pack form (nt2cuda/expr.cuh, nt2cuda/trig.cuh).
// Included by capi_trigx_f32.cu and capi_trigx_f64.cu, one element type each.
#pragma once
#include <cuda_runtime.h>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/launch.cuh"

namespace nt2cuda {
namespace detail_capi {

namespace {

template <class Tag, class... C> node<Tag, C...> nd(C... c) { return node<Tag, C...>{c...}; }

template <bool F, class E, class T> nt2cuda_status run_e(const E& e, T* y, size_t n, nt2cuda_stream s)
{
  auto p = make_prog(assign<T, E>{y, e});
  return launch_status(transform<F>(p, n, as_stream(s), "trig"));
}

template <class Tag, bool SIMD> struct pick { using type = Tag; };
template <class Tag> struct pick<Tag, true> { using type = tag::simd128_<Tag>; };

// csc, sec, cscpi, secpi, cscd, cot, tanpi, cotpi, sind, cosd, tand, cotd, secd: the
// reduced node in the form SIMD selects
template <bool F, bool SIMD, class T> nt2cuda_status recip_impl(int op, const T* x, T* y, size_t n, nt2cuda_stream s)
{
  const term<T> X{x};
  using Sin = typename pick<tag::sin_, SIMD>::type;
  using Cos = typename pick<tag::cos_, SIMD>::type;
  using Sinpi = typename pick<tag::sinpi_, SIMD>::type;
  using Cospi = typename pick<tag::cospi_, SIMD>::type;
  switch (op) {
    case NT2CUDA_OP_CSC: return run_e<F>(nd<tag::rec_>(nd<Sin>(X)), y, n, s);
    case NT2CUDA_OP_SEC: return run_e<F>(nd<tag::rec_>(nd<Cos>(X)), y, n, s);
    case NT2CUDA_OP_CSCPI: return run_e<F>(nd<tag::cscpi_nan_>(X, nd<tag::rec_>(nd<Sinpi>(X))), y, n, s);
    case NT2CUDA_OP_SECPI: return run_e<F>(nd<tag::secpi_nan_>(X, nd<tag::rec_>(nd<Cospi>(X))), y, n, s);
    case NT2CUDA_OP_CSCD: {
      const auto Y = nd<tag::oneo_180_mul_>(X);
      return run_e<F>(nd<tag::cscpi_nan_>(Y, nd<tag::rec_>(nd<Sinpi>(Y))), y, n, s);
    }
    case NT2CUDA_OP_COT: return run_e<F>(nd<typename pick<tag::cot_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_TANPI: return run_e<F>(nd<typename pick<tag::tanpi_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_COTPI: return run_e<F>(nd<typename pick<tag::cotpi_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_SIND: return run_e<F>(nd<typename pick<tag::sind_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_COSD: return run_e<F>(nd<typename pick<tag::cosd_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_TAND: return run_e<F>(nd<typename pick<tag::tand_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_COTD: return run_e<F>(nd<typename pick<tag::cotd_, SIMD>::type>(X), y, n, s);
    case NT2CUDA_OP_SINC:
      return run_e<F>(nd<tag::sinc_fix_>(X, nd<tag::divides_>(nd<Sin>(X), X)), y, n, s);
    case NT2CUDA_OP_SINCPI:
      return run_e<F>(nd<tag::sinc_fix_>(X, nd<tag::invpi_mul_>(nd<tag::divides_>(nd<Sinpi>(X), X))), y, n, s);
    case NT2CUDA_OP_SECD:
      return run_e<F>(nd<tag::rec_>(nd<tag::nan_if_zero_>(nd<typename pick<tag::cosd_, SIMD>::type>(X))), y, n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}

// the inverse functors and the unit conversions: no pack dependence
template <bool F, class T> nt2cuda_status inv_impl(int op, const T* x, T* y, size_t n, nt2cuda_stream s)
{
  const term<T> X{x};
  const auto R = nd<tag::rec_>(X);
  switch (op) {
    case NT2CUDA_OP_INDEG: return run_e<F>(nd<tag::indeg_>(X), y, n, s);
    case NT2CUDA_OP_INRAD: return run_e<F>(nd<tag::inrad_>(X), y, n, s);
    case NT2CUDA_OP_ACOT: return run_e<F>(nd<tag::atan_>(R), y, n, s);
    case NT2CUDA_OP_ASIND: return run_e<F>(nd<tag::indeg_>(nd<tag::asin_>(X)), y, n, s);
    case NT2CUDA_OP_ACOSD: return run_e<F>(nd<tag::indeg_>(nd<tag::acos_>(X)), y, n, s);
    case NT2CUDA_OP_ATAND: return run_e<F>(nd<tag::indeg_>(nd<tag::atan_>(X)), y, n, s);
    case NT2CUDA_OP_ASINPI: return run_e<F>(nd<tag::invpi_mul_>(nd<tag::asin_>(X)), y, n, s);
    case NT2CUDA_OP_ACOSPI: return run_e<F>(nd<tag::invpi_mul_>(nd<tag::acos_>(X)), y, n, s);
    case NT2CUDA_OP_ATANPI: return run_e<F>(nd<tag::invpi_mul_>(nd<tag::atan_>(X)), y, n, s);
    case NT2CUDA_OP_ACSC: return run_e<F>(nd<tag::asin_>(R), y, n, s);
    case NT2CUDA_OP_ACSCD: return run_e<F>(nd<tag::indeg_>(nd<tag::asin_>(R)), y, n, s);
    case NT2CUDA_OP_ASEC: return run_e<F>(nd<tag::pio2_minus_>(nd<tag::asin_>(R)), y, n, s);
    case NT2CUDA_OP_ASECD: return run_e<F>(nd<tag::indeg_>(nd<tag::pio2_minus_>(nd<tag::asin_>(R))), y, n, s);
    case NT2CUDA_OP_FAST_SIN: return run_e<F>(nd<tag::fast_<0, 0>>(X), y, n, s);
    case NT2CUDA_OP_FAST_COS: return run_e<F>(nd<tag::fast_<1, 0>>(X), y, n, s);
    case NT2CUDA_OP_FAST_TAN: return run_e<F>(nd<tag::fast_<2, 0>>(X), y, n, s);
    case NT2CUDA_OP_FAST_COT: return run_e<F>(nd<tag::fast_<3, 0>>(X), y, n, s);
    case NT2CUDA_OP_FAST_SINPI: return run_e<F>(nd<tag::fast_<0, 1>>(X), y, n, s);
    case NT2CUDA_OP_FAST_COSPI: return run_e<F>(nd<tag::fast_<1, 1>>(X), y, n, s);
    case NT2CUDA_OP_FAST_TANPI: return run_e<F>(nd<tag::fast_<2, 1>>(X), y, n, s);
    case NT2CUDA_OP_FAST_COTPI: return run_e<F>(nd<tag::fast_<3, 1>>(X), y, n, s);
    case NT2CUDA_OP_FAST_SIND: return run_e<F>(nd<tag::fast_<0, 2>>(X), y, n, s);
    case NT2CUDA_OP_FAST_COSD: return run_e<F>(nd<tag::fast_<1, 2>>(X), y, n, s);
    case NT2CUDA_OP_FAST_TAND: return run_e<F>(nd<tag::fast_<2, 2>>(X), y, n, s);
    case NT2CUDA_OP_FAST_COTD: return run_e<F>(nd<tag::fast_<3, 2>>(X), y, n, s);
    case NT2CUDA_OP_PROPER_TANPI: return run_e<F>(nd<tag::proper_tanpi_>(X), y, n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}

// tie(s, c) = sincos(x) and its pi, degree and fast forms: two assigns of one statement
template <bool F, class ES, class EC, class T>
nt2cuda_status run_pair(const ES& es, const EC& ec, T* s_out, T* c_out, size_t n, nt2cuda_stream s)
{
  auto p = make_prog(assign<T, ES>{s_out, es}, assign<T, EC>{c_out, ec});
  return launch_status(transform<F>(p, n, as_stream(s), "trig"));
}
template <bool F, bool SIMD, class T>
nt2cuda_status sincos_impl(int form, const T* x, T* so, T* co, size_t n, nt2cuda_stream s)
{
  const term<T> X{x};
  switch (form) {
    case NT2CUDA_SINCOS:
      return run_pair<F>(nd<typename pick<tag::sin_, SIMD>::type>(X), nd<typename pick<tag::cos_, SIMD>::type>(X), so, co, n, s);
    case NT2CUDA_SINCOSPI:
      return run_pair<F>(nd<typename pick<tag::sinpi_, SIMD>::type>(X), nd<typename pick<tag::cospi_, SIMD>::type>(X), so, co,
                         n, s);
    case NT2CUDA_SINCOSD:
      return run_pair<F>(nd<typename pick<tag::sind_, SIMD>::type>(X), nd<typename pick<tag::cosd_, SIMD>::type>(X), so, co,
                         n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}
template <bool F, class T> nt2cuda_status fast_sincos_impl(int form, const T* x, T* so, T* co, size_t n, nt2cuda_stream s)
{
  const term<T> X{x};
  switch (form) {
    case NT2CUDA_FAST_SINCOS: return run_pair<F>(nd<tag::fast_<0, 0>>(X), nd<tag::fast_<1, 0>>(X), so, co, n, s);
    case NT2CUDA_FAST_SINCOSPI: return run_pair<F>(nd<tag::fast_<0, 1>>(X), nd<tag::fast_<1, 1>>(X), so, co, n, s);
    case NT2CUDA_FAST_SINCOSD: return run_pair<F>(nd<tag::fast_<0, 2>>(X), nd<tag::fast_<1, 2>>(X), so, co, n, s);
    case NT2CUDA_SINHCOSH: return run_pair<F>(nd<tag::sinh_>(X), nd<tag::cosh_>(X), so, co, n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}
template <class T> nt2cuda_status sincos_dispatch(int form, const T* x, T* so, T* co, size_t n, bool fused, bool simd,
                                                  nt2cuda_stream s)
{
  if (form >= NT2CUDA_FAST_SINCOS)
    return fused ? fast_sincos_impl<true>(form, x, so, co, n, s) : fast_sincos_impl<false>(form, x, so, co, n, s);
  if (fused) return simd ? sincos_impl<true, true>(form, x, so, co, n, s) : sincos_impl<true, false>(form, x, so, co, n, s);
  return simd ? sincos_impl<false, true>(form, x, so, co, n, s) : sincos_impl<false, false>(form, x, so, co, n, s);
}

// The functors with a reduction are compiled in their own translation units, one
// per form (capi_trigx_fwd_*.cu: scalar form, capi_trigx_fwd128_*.cu: 128-bit form).
template <class T> nt2cuda_status trigx_dispatch(int op, const T* x, T* y, size_t n, bool fused, bool simd,
                                                 nt2cuda_stream s)
{
  const bool packless = (op >= NT2CUDA_OP_INDEG && op <= NT2CUDA_OP_ASECD) ||
                        (op >= NT2CUDA_OP_FAST_SIN && op <= NT2CUDA_OP_FAST_COTD) || op == NT2CUDA_OP_PROPER_TANPI;
  if (packless) return fused ? inv_impl<true>(op, x, y, n, s) : inv_impl<false>(op, x, y, n, s);
  return simd ? trigx_fwd_simd128(op, x, y, n, fused, s) : trigx_fwd_scalar(op, x, y, n, fused, s);
}

}  // namespace

}  // namespace detail_capi
}  // namespace nt2cuda
