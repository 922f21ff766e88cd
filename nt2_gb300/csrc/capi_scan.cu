// capi_scan.cu -- C-ABI entry points of the cumulative functions (cumsum,
// cumprod, cummax, cummin) through inner_scan / outer_scan (nt2cuda/scan.cuh).
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.cuh"
#include "nt2cuda/launch.cuh"
#include "nt2cuda/scan_launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;
using nt2cuda::fold::state_of;

namespace {

template <class T>
nt2cuda_status scan_impl(int op, const T* A, size_t rows, size_t cols, int dim, T* out, int flags, cudaStream_t s)
{
  using namespace fold;
  if ((dim != 1 && dim != 2) || (rows && cols && (!A || !out))) return NT2CUDA_ERR_ARG;
  const size_t bytes = rows * cols * sizeof(T);
  const uintptr_t a = (uintptr_t)A, o = (uintptr_t)out;
  if (a != o && a < o + bytes && o < a + bytes) return NT2CUDA_ERR_ALIAS;   // in place is fine
  const bool comp = sizeof(T) == 4 && !(flags & NT2CUDA_RED_PLAIN);
  cudaError_t e;
  switch (op) {
    case NT2CUDA_SCAN_SUM:
      e = comp ? scan::scan_dim<op_sum<true>, T>(A, out, rows, cols, dim, s) : scan::scan_dim<op_sum<false>, T>(A, out, rows, cols, dim, s);
      break;
    case NT2CUDA_SCAN_PROD: e = scan::scan_dim<op_val<2>, T>(A, out, rows, cols, dim, s); break;
    case NT2CUDA_SCAN_MAX: e = scan::scan_dim<op_val<3>, T>(A, out, rows, cols, dim, s); break;
    case NT2CUDA_SCAN_MIN: e = scan::scan_dim<op_val<4>, T>(A, out, rows, cols, dim, s); break;
    default: return NT2CUDA_ERR_ARG;
  }
  return launch_status(e);
}

}  // namespace

extern "C" {

nt2cuda_status nt2cuda_scan_f32(int op, const float* A, size_t rows, size_t cols, int dim, float* out, int flags,
                                nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  return scan_impl<float>(op, A, rows, cols, dim, out, flags, as_stream(s));
}

nt2cuda_status nt2cuda_scan_f64(int op, const double* A, size_t rows, size_t cols, int dim, double* out, int flags,
                                nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  return scan_impl<double>(op, A, rows, cols, dim, out, flags, as_stream(s));
}

nt2cuda_status nt2cuda_wait_timeouts(unsigned long long* count)
{
  if (!count) return NT2CUDA_ERR_ARG;
  return from_cuda(scan::wait_timeouts(count));
}

nt2cuda_status nt2cuda_selftest_wait_timeout(nt2cuda_stream s)
{
  unsigned failed = 0;
  const nt2cuda_status st = from_cuda(scan::selftest_wait_timeout(as_stream(s), &failed));
  if (st != NT2CUDA_OK) return st;
  return failed ? NT2CUDA_ERR_TIMEOUT : NT2CUDA_OK;
}

}  // extern "C"
