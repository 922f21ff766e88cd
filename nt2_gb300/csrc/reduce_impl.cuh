// reduce_impl.cuh -- the reductions of NT2's reduction module on the fold
// kernels: sum, asum1, asum2, norm2, mean, var, stdev, max, min, prod (one
// value per output) and all, any, none (logical outputs), along dimension 1
// (one value per column, inner_fold), dimension 2 (one value per row,
// outer_fold) or over the whole table (dim 0, NT2's global* functions,
// nt2/core/functions/global.hpp:19-31).
//   asum1(A,d) = sum(abs(A),d)             nt2/core/functions/expr/asum1.hpp
//   asum2(A,d) = sum(sqr_abs(A),d)         nt2/core/functions/expr/asum2.hpp
//   norm2(A,d) = sqrt(asum2(A,d))          nt2/core/functions/expr/norm2.hpp
//   mean(A,d)  = rec(n) * sum(A,d)         nt2/core/functions/expr/mean.hpp
//   var(A,w,d) = f * asum2(center(A,d),d)  nt2/core/functions/expr/var.hpp
//   stdev      = realsqrt(var)             nt2/core/functions/expr/stdev.hpp
//   max/min/prod/all/any/none: boost/simd/reduction/functions/{maximum,minimum,prod,all,any,none}.hpp
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/fold.cuh"
#include "nt2cuda/fold_launch.cuh"

namespace nt2cuda {
namespace detail_capi {

template <class Op, class T, class E>
cudaError_t fold_dim(const E& e, size_t rows, size_t cols, int dim, fold::out_of<Op, T>* out, cudaStream_t s)
{
  switch (dim) {
    case 0: return fold::inner_fold<Op, T>(e, rows * cols, 1, out, s);
    case 1: return fold::inner_fold<Op, T>(e, rows, cols, out, s);
    default: return fold::outer_fold<Op, T>(e, rows, cols, out, s);
  }
}

template <class T>
nt2cuda_status reduce_impl(int op, const T* A, size_t rows, size_t cols, int dim, T* out, int flags, cudaStream_t s)
{
  using namespace fold;
  if (dim < 0 || dim > 2 || !out || (rows && cols && !A)) return NT2CUDA_ERR_ARG;
  // FP64 tables accumulate plainly (the FP64 sum is the reference's own precision)
  const bool comp = sizeof(T) == 4 && !(flags & NT2CUDA_RED_PLAIN);
  const bool w1 = (flags & NT2CUDA_RED_VAR_N) != 0;
  const term<T> x{A};
  const node<tag::abs_, term<T>> ax{x};
  const node<tag::sqr_, term<T>> sx{x};
  cudaError_t e;
  switch (op) {
    case NT2CUDA_RED_SUM:
      e = comp ? fold_dim<op_sum<true>, T>(x, rows, cols, dim, out, s) : fold_dim<op_sum<false>, T>(x, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_ASUM1:
      e = comp ? fold_dim<op_sum<true>, T>(ax, rows, cols, dim, out, s) : fold_dim<op_sum<false>, T>(ax, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_ASUM2:
      e = comp ? fold_dim<op_sum<true>, T>(sx, rows, cols, dim, out, s) : fold_dim<op_sum<false>, T>(sx, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_NORM2:
      e = comp ? fold_dim<op_sum<true, FIN_SQRT>, T>(sx, rows, cols, dim, out, s)
               : fold_dim<op_sum<false, FIN_SQRT>, T>(sx, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_MEAN:
      e = comp ? fold_dim<op_sum<true, FIN_MEAN>, T>(x, rows, cols, dim, out, s)
               : fold_dim<op_sum<false, FIN_MEAN>, T>(x, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_VAR:
      e = w1 ? fold_dim<op_moments<true, false>, T>(x, rows, cols, dim, out, s)
             : fold_dim<op_moments<false, false>, T>(x, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_STDEV:
      e = w1 ? fold_dim<op_moments<true, true>, T>(x, rows, cols, dim, out, s)
             : fold_dim<op_moments<false, true>, T>(x, rows, cols, dim, out, s);
      break;
    case NT2CUDA_RED_MAX: e = fold_dim<op_val<0>, T>(x, rows, cols, dim, out, s); break;
    case NT2CUDA_RED_MIN: e = fold_dim<op_val<1>, T>(x, rows, cols, dim, out, s); break;
    case NT2CUDA_RED_PROD: e = fold_dim<op_val<2>, T>(x, rows, cols, dim, out, s); break;
    default: return NT2CUDA_ERR_ARG;
  }
  return launch_status(e);
}

template <class T>
nt2cuda_status reduce_logical_impl(int op, const T* A, size_t rows, size_t cols, int dim, uint8_t* out,
                                   cudaStream_t s)
{
  using namespace fold;
  if (dim < 0 || dim > 2 || !out || (rows && cols && !A)) return NT2CUDA_ERR_ARG;
  const term<T> x{A};
  cudaError_t e;
  switch (op) {
    case NT2CUDA_RED_ALL: e = fold_dim<op_logic<false>, T>(x, rows, cols, dim, out, s); break;
    case NT2CUDA_RED_ANY: e = fold_dim<op_logic<true>, T>(x, rows, cols, dim, out, s); break;
    case NT2CUDA_RED_NONE: e = fold_dim<op_logic<true, true>, T>(x, rows, cols, dim, out, s); break;
    default: return NT2CUDA_ERR_ARG;
  }
  return launch_status(e);
}

}  // namespace detail_capi
}  // namespace nt2cuda
