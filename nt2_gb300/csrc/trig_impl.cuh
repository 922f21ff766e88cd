// trig_impl.cuh -- the trigonometric and hyperbolic functors of
// nt2cuda_map_f32/f64 (sin, cos, tan, sinpi, cospi in NT2's scalar form or its
// 128-bit SIMD form; asin, acos, atan; sinh, cosh, tanh) and the binary
// atan2 and pow, lowered onto the elementwise transform (nt2cuda/trig.cuh,
// nt2cuda/math.cuh).  Included by
// capi_trig_f32.cu and capi_trig_f64.cu, one element type each, which the
// build compiles in parallel.
#pragma once
#include <cuda_runtime.h>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/launch.cuh"

namespace nt2cuda {
namespace detail_capi {

namespace {

template <bool F, class Tag, class T> nt2cuda_status run_trig(const T* x, T* y, size_t n, nt2cuda_stream s)
{
  auto p = make_prog(assign<T, node<Tag, term<T>>>{y, node<Tag, term<T>>{term<T>{x}}});
  // two groups in flight per thread (the default): 10-15% faster than one on
  // 2^24 floats, although two of the 128-bit kernels then spill a few words
  return launch_status(transform<F>(p, n, as_stream(s), "trig"));
}

template <class Tag, bool SIMD> struct form { using type = Tag; };
template <class Tag> struct form<Tag, true> { using type = tag::simd128_<Tag>; };

template <bool F, bool SIMD, class T> nt2cuda_status trig_impl(int op, const T* x, T* y, size_t n, nt2cuda_stream s)
{
  switch (op) {
    case NT2CUDA_OP_SIN: return run_trig<F, typename form<tag::sin_, SIMD>::type>(x, y, n, s);
    case NT2CUDA_OP_COS: return run_trig<F, typename form<tag::cos_, SIMD>::type>(x, y, n, s);
    case NT2CUDA_OP_TAN: return run_trig<F, typename form<tag::tan_, SIMD>::type>(x, y, n, s);
    case NT2CUDA_OP_SINPI: return run_trig<F, typename form<tag::sinpi_, SIMD>::type>(x, y, n, s);
    case NT2CUDA_OP_COSPI: return run_trig<F, typename form<tag::cospi_, SIMD>::type>(x, y, n, s);
    // the inverse functions do not depend on the pack: one form
    case NT2CUDA_OP_ASIN: return SIMD ? NT2CUDA_ERR_ARG : run_trig<F, tag::asin_>(x, y, n, s);
    case NT2CUDA_OP_ACOS: return SIMD ? NT2CUDA_ERR_ARG : run_trig<F, tag::acos_>(x, y, n, s);
    case NT2CUDA_OP_ATAN: return SIMD ? NT2CUDA_ERR_ARG : run_trig<F, tag::atan_>(x, y, n, s);
    case NT2CUDA_OP_SINH: return SIMD ? NT2CUDA_ERR_ARG : run_trig<F, tag::sinh_>(x, y, n, s);
    case NT2CUDA_OP_COSH: return SIMD ? NT2CUDA_ERR_ARG : run_trig<F, tag::cosh_>(x, y, n, s);
    case NT2CUDA_OP_TANH: return SIMD ? NT2CUDA_ERR_ARG : run_trig<F, tag::tanh_>(x, y, n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}

template <class T> nt2cuda_status dispatch(int op, const T* x, T* y, size_t n, bool fused, bool simd, nt2cuda_stream s)
{
  if (op >= NT2CUDA_OP_ASIN) simd = false;   // no pack dependence: the flag changes nothing
  if (fused) return simd ? trig_impl<true, true>(op, x, y, n, s) : trig_impl<true, false>(op, x, y, n, s);
  return simd ? trig_impl<false, true>(op, x, y, n, s) : trig_impl<false, false>(op, x, y, n, s);
}

template <class Tag, class T>
nt2cuda_status binary_impl(const T* a0, const T* a1, T* y, size_t n, bool fused, nt2cuda_stream s)
{
  using N = node<Tag, term<T>, term<T>>;
  auto p = make_prog(assign<T, N>{y, N{term<T>{a0}, term<T>{a1}}});
  return launch_status(fused ? transform<true>(p, n, as_stream(s), "trig") : transform<false>(p, n, as_stream(s), "trig"));
}

}  // namespace

}  // namespace detail_capi
}  // namespace nt2cuda
