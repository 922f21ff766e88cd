// expfam_impl.cuh -- the rest of NT2's exponential family on the elementwise
// transform: the unary ops NT2CUDA_OP_CBRT..NT2CUDA_OP_REALLOG of
// nt2cuda_map_f32/f64 and the binary functors of nt2cuda_map2_f32/f64
// (nt2cuda/math.cuh holds the functors).  Included by capi_expfam_f32.cu and
// capi_expfam_f64.cu, one element type each.
#pragma once
#include <cuda_runtime.h>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/launch.cuh"

namespace nt2cuda {
namespace detail_capi {

namespace {

template <bool F, class Tag, class T> nt2cuda_status run_unary(const T* x, T* y, size_t n, nt2cuda_stream s)
{
  auto p = make_prog(assign<T, node<Tag, term<T>>>{y, node<Tag, term<T>>{term<T>{x}}});
  return launch_status(transform<F>(p, n, as_stream(s), "map"));
}

template <bool F, class E, class T> nt2cuda_status run_tree(const E& e, T* y, size_t n, nt2cuda_stream s)
{
  auto p = make_prog(assign<T, E>{y, e});
  return launch_status(transform<F>(p, n, as_stream(s), "map"));
}

template <bool F, class T> nt2cuda_status expfam_impl(int op, const T* x, T* y, size_t n, nt2cuda_stream s)
{
  switch (op) {
    case NT2CUDA_OP_CBRT: return run_unary<F, tag::cbrt_>(x, y, n, s);
    case NT2CUDA_OP_SQRT1PM1: return run_unary<F, tag::sqrt1pm1_>(x, y, n, s);
    case NT2CUDA_OP_EXPRECNEG: return run_unary<F, tag::exprecneg_>(x, y, n, s);
    case NT2CUDA_OP_EXPRECNEGC: return run_unary<F, tag::exprecnegc_>(x, y, n, s);
    case NT2CUDA_OP_EXPX2: return run_unary<F, tag::expx2_>(x, y, n, s);
    // NT2's assertion (x >= 0) is a debug check; the value is sqrt's / log's
    case NT2CUDA_OP_REALSQRT: return run_unary<F, tag::sqrt_>(x, y, n, s);
    case NT2CUDA_OP_REALLOG: return run_unary<F, tag::log_>(x, y, n, s);
    case NT2CUDA_OP_ATANH: return run_unary<F, tag::atanh_>(x, y, n, s);
    case NT2CUDA_OP_ACOSH: return run_unary<F, tag::acosh_>(x, y, n, s);
    case NT2CUDA_OP_SECH: return run_tree<F>(node<tag::rec_, node<tag::cosh_, term<T>>>{{term<T>{x}}}, y, n, s);
    case NT2CUDA_OP_CSCH: return run_tree<F>(node<tag::rec_, node<tag::sinh_, term<T>>>{{term<T>{x}}}, y, n, s);
    case NT2CUDA_OP_ACOTH: return run_tree<F>(node<tag::atanh_, node<tag::rec_, term<T>>>{{term<T>{x}}}, y, n, s);
    case NT2CUDA_OP_ASECH: return run_tree<F>(node<tag::acosh_, node<tag::rec_, term<T>>>{{term<T>{x}}}, y, n, s);
    case NT2CUDA_OP_ASINH: return run_unary<F, tag::asinh_>(x, y, n, s);
    case NT2CUDA_OP_COTH: return run_unary<F, tag::coth_>(x, y, n, s);
    case NT2CUDA_OP_SINHC: return run_unary<F, tag::sinhc_>(x, y, n, s);
    case NT2CUDA_OP_ACSCH: return run_tree<F>(node<tag::asinh_, node<tag::rec_, term<T>>>{{term<T>{x}}}, y, n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}

template <bool F, class Tag, class T>
nt2cuda_status run_binary(const T* a0, const T* a1, T* y, size_t n, nt2cuda_stream s)
{
  using N = node<Tag, term<T>, term<T>>;
  auto p = make_prog(assign<T, N>{y, N{term<T>{a0}, term<T>{a1}}});
  return launch_status(transform<F>(p, n, as_stream(s), "map2"));
}

template <bool F, class T> nt2cuda_status map2_impl(int op, const T* a0, const T* a1, T* y, size_t n, nt2cuda_stream s)
{
  switch (op) {
    case NT2CUDA_OP2_POW_ABS: return run_binary<F, tag::pow_abs_>(a0, a1, y, n, s);
    case NT2CUDA_OP2_LOGSPACE_ADD: return run_binary<F, tag::logspace_add_>(a0, a1, y, n, s);
    case NT2CUDA_OP2_LOGSPACE_SUB: return run_binary<F, tag::logspace_sub_>(a0, a1, y, n, s);
    case NT2CUDA_OP2_EXPX2: return run_binary<F, tag::expx2s_>(a0, a1, y, n, s);
    case NT2CUDA_OP2_ATAN2D: return run_binary<F, tag::atan2d_>(a0, a1, y, n, s);
    case NT2CUDA_OP2_NBD_ATAN2: return run_binary<F, tag::nbd_atan2_>(a0, a1, y, n, s);
    case NT2CUDA_OP2_HYPOT: return run_binary<F, tag::hypot_>(a0, a1, y, n, s);
    default: return NT2CUDA_ERR_ARG;
  }
}

}  // namespace

}  // namespace detail_capi
}  // namespace nt2cuda
