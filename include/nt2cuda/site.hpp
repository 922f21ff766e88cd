// nt2cuda/site.hpp -- the three operations of NT2's evaluation site, on
// lowered trees: transform_, inner_fold_ and outer_fold_.
//
// NT2's backends implement these overloads for their site
// (modules/arch/shared_memory/include/nt2/core/functions/shared_memory/transform.hpp:26-50,
//  .../shared_memory/inner_fold.hpp:24-63, .../shared_memory/outer_fold.hpp:22-51);
// nt2/sdk/cuda/eval.hpp registers the GPU ones with Boost.Dispatch and
// forwards here.  Nothing in this header needs Boost: a statement arrives as
// a tree that tree_access<> can read (table_lowering.hpp), is lowered to one
// nt2cuda expression type and runs as one fused kernel (transform) or one
// fold launch.  Every call returns with its results in the output table, as
// NT2's operator= does, and reports failure as a cudaError_t.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <type_traits>
#include "nt2cuda/fold_launch.cuh"
#include "nt2cuda/launch.cuh"
#include "nt2cuda/table_lowering.hpp"

namespace nt2cuda {
namespace site {

// Per host thread: the stream the site's kernels run on, NT2's fused
// fma/fnms (off: NT2's generic a*b+c rounded twice), and compensated FP32 sums.
struct site_settings {
  cudaStream_t stream = nullptr;
  bool fused = false;
  bool compensated = true;
};
inline site_settings& settings()
{
  static thread_local site_settings s;
  return s;
}

// out[begin, begin + size) = in[begin, begin + size).  `out` points at the
// first element of the output table.
template <class T, class In> cudaError_t transform(T* out, In& in, size_t begin, size_t size)
{
  static_assert(lowering::lowerable<In>::value, "statement has a functor or leaf without a device form");
  if (size == 0) return cudaSuccess;
  auto e = lowering::lower<T>(in, begin);
  auto p = make_prog(assign<T, decltype(e)>{out + begin, e});
  const site_settings& st = settings();
  cudaError_t r = st.fused ? nt2cuda::transform<true>(p, size, st.stream) : nt2cuda::transform<false>(p, size, st.stream);
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r == cudaSuccess) r = cudaStreamSynchronize(st.stream);
  return r;
}

// The fold operation of an NT2 reduction tag (lowering::fold_of).
template <int Kind, bool Comp> struct fold_op;
template <bool Comp> struct fold_op<lowering::FOLD_SUM, Comp> { using type = fold::op_sum<Comp>; };
template <bool Comp> struct fold_op<lowering::FOLD_MAX, Comp> { using type = fold::op_val<0>; };
template <bool Comp> struct fold_op<lowering::FOLD_MIN, Comp> { using type = fold::op_val<1>; };
template <bool Comp> struct fold_op<lowering::FOLD_PROD, Comp> { using type = fold::op_val<2>; };

// Reductions whose result has the element type (sum, prod, maximum, minimum).
template <int Kind> struct site_fold : std::integral_constant<bool, Kind == lowering::FOLD_SUM || Kind == lowering::FOLD_PROD ||
                                                                     Kind == lowering::FOLD_MAX || Kind == lowering::FOLD_MIN> {};

// inner_fold: in viewed as (inner, outer) column-major; out[j] = fold over i
// of in(i, j) (reduction/run.hpp:72-79 reshapes to of_size(inner, hi)).
template <int Kind, class T, class In> cudaError_t inner_fold(T* out, In& in, size_t inner, size_t outer)
{
  static_assert(site_fold<Kind>::value, "reduction without a device form");
  if (inner == 0 || outer == 0) return cudaSuccess;
  auto e = lowering::lower<T>(in, 0);
  const site_settings& st = settings();
  cudaError_t r = (std::is_same<T, float>::value && st.compensated)
                      ? fold::inner_fold<typename fold_op<Kind, true>::type, T>(e, inner, outer, out, st.stream)
                      : fold::inner_fold<typename fold_op<Kind, false>::type, T>(e, inner, outer, out, st.stream);
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r == cudaSuccess) r = cudaStreamSynchronize(st.stream);
  return r;
}

// outer_fold: in viewed as (lo, inner, hi); out(l, k) = fold over m of
// in(l, m, k) (reduction/run.hpp:82-88 reshapes to of_size(lo, inner, hi)).
// Each of the hi slabs is one row fold of a lo x inner table.
template <int Kind, class T, class In> cudaError_t outer_fold(T* out, In& in, size_t lo, size_t inner, size_t hi)
{
  static_assert(site_fold<Kind>::value, "reduction without a device form");
  if (lo == 0 || inner == 0 || hi == 0) return cudaSuccess;
  const site_settings& st = settings();
  cudaError_t r = cudaSuccess;
  for (size_t k = 0; k < hi && r == cudaSuccess; ++k) {
    auto e = lowering::lower<T>(in, k * lo * inner);
    r = (std::is_same<T, float>::value && st.compensated)
            ? fold::outer_fold<typename fold_op<Kind, true>::type, T>(e, lo, inner, out + k * lo, st.stream)
            : fold::outer_fold<typename fold_op<Kind, false>::type, T>(e, lo, inner, out + k * lo, st.stream);
  }
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r == cudaSuccess) r = cudaStreamSynchronize(st.stream);
  return r;
}

}  // namespace site
}  // namespace nt2cuda
