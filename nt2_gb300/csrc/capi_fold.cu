// capi_fold.cu -- C-ABI entry points for the inner_fold / outer_fold site
// overloads: globalsum, dot (globalsum of X*Y), sum(A,1) and sum(A,2).
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/fold.cuh"
#include "nt2cuda/fold_launch.cuh"
#include "nt2cuda/fold_tma.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;
using nt2cuda::fold::acc;

extern "C" {

nt2cuda_status nt2cuda_globalsum_f32(const float* x, size_t n, float* out, int compensated, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((n && !x) || !out) return NT2CUDA_ERR_ARG;
  term<float> e{x};
  return launch_status(compensated ? nt2cuda::fold::inner_fold<fold::op_sum<true>, float>(e, n, 1, out, as_stream(s))
                     : nt2cuda::fold::inner_fold<fold::op_sum<false>, float>(e, n, 1, out, as_stream(s)));
}

nt2cuda_status nt2cuda_dot_f32(const float* x, const float* y, size_t n, float* out, int compensated,
                               nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((n && (!x || !y)) || !out) return NT2CUDA_ERR_ARG;
  node<tag::multiplies_, term<float>, term<float>> e{term<float>{x}, term<float>{y}};
  return launch_status(compensated ? nt2cuda::fold::inner_fold<fold::op_sum<true>, float>(e, n, 1, out, as_stream(s))
                     : nt2cuda::fold::inner_fold<fold::op_sum<false>, float>(e, n, 1, out, as_stream(s)));
}

nt2cuda_status nt2cuda_globalsum_f64(const double* x, size_t n, double* out, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((n && !x) || !out) return NT2CUDA_ERR_ARG;
  return launch_status(nt2cuda::fold::inner_fold<fold::op_sum<false>, double>(term<double>{x}, n, 1, out, as_stream(s)));
}

nt2cuda_status nt2cuda_dot_f64(const double* x, const double* y, size_t n, double* out, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((n && (!x || !y)) || !out) return NT2CUDA_ERR_ARG;
  node<tag::multiplies_, term<double>, term<double>> e{term<double>{x}, term<double>{y}};
  return launch_status(nt2cuda::fold::inner_fold<fold::op_sum<false>, double>(e, n, 1, out, as_stream(s)));
}

nt2cuda_status nt2cuda_sum_inner_f32(const float* A, size_t rows, size_t cols, float* out, int compensated,
                                     nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((rows && cols && !A) || !out) return NT2CUDA_ERR_ARG;
  term<float> e{A};
  return launch_status(compensated ? nt2cuda::fold::inner_fold<fold::op_sum<true>, float>(e, rows, cols, out, as_stream(s))
                     : nt2cuda::fold::inner_fold<fold::op_sum<false>, float>(e, rows, cols, out, as_stream(s)));
}

nt2cuda_status nt2cuda_sum_inner_f64(const double* A, size_t rows, size_t cols, double* out, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((rows && cols && !A) || !out) return NT2CUDA_ERR_ARG;
  return launch_status(nt2cuda::fold::inner_fold<fold::op_sum<false>, double>(term<double>{A}, rows, cols, out, as_stream(s)));
}

nt2cuda_status nt2cuda_sum_outer_f32(const float* A, size_t rows, size_t cols, float* out, int compensated,
                                     nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((rows && cols && !A) || !out) return NT2CUDA_ERR_ARG;
  term<float> e{A};
  return launch_status(compensated ? nt2cuda::fold::outer_fold<fold::op_sum<true>, float>(e, rows, cols, out, as_stream(s))
                     : nt2cuda::fold::outer_fold<fold::op_sum<false>, float>(e, rows, cols, out, as_stream(s)));
}

nt2cuda_status nt2cuda_sum_outer_f64(const double* A, size_t rows, size_t cols, double* out, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if ((rows && cols && !A) || !out) return NT2CUDA_ERR_ARG;
  return launch_status(nt2cuda::fold::outer_fold<fold::op_sum<false>, double>(term<double>{A}, rows, cols, out, as_stream(s)));
}

nt2cuda_status nt2cuda_selftest_fold_timeout(const float* A, size_t rows, size_t cols, float* out, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (!A || !out || !cols || ((uintptr_t)A & 15u) || rows % 4 || rows <= (size_t)fold::inner_tile<float>() * 16)
    return NT2CUDA_ERR_ARG;
  unsigned long long before = 0, after = 0;
  cudaError_t e = fold::read_fold_wait_timeouts(&before);
  if (e == cudaSuccess)
    e = fold::inner_fold_tma<fold::op_sum<true>, float>(A, nullptr, rows, cols, out, as_stream(s), 0, 1u << 12);
  if (e == cudaSuccess) e = cudaStreamSynchronize(as_stream(s));
  if (e == cudaSuccess) e = fold::read_fold_wait_timeouts(&after);
  if (e != cudaSuccess) return from_cuda(e);
  return after > before ? NT2CUDA_ERR_TIMEOUT : NT2CUDA_OK;
}

nt2cuda_status nt2cuda_set_fold_path(int path)
{
  if (path < 0 || path > 2) return NT2CUDA_ERR_ARG;
  nt2cuda::fold::fold_path().store(path);
  return NT2CUDA_OK;
}

}  // extern "C"
