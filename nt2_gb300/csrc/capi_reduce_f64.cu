// capi_reduce_f64.cu -- C-ABI entry points of the FP64 reductions (reduce_impl.cuh).
#include "reduce_impl.cuh"

using namespace nt2cuda::detail_capi;

extern "C" {

nt2cuda_status nt2cuda_reduce_f64(int op, const double* A, size_t rows, size_t cols, int dim, double* out, int flags,
                                  nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  return reduce_impl<double>(op, A, rows, cols, dim, out, flags, as_stream(s));
}

nt2cuda_status nt2cuda_reduce_logical_f64(int op, const double* A, size_t rows, size_t cols, int dim, uint8_t* out,
                                          nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  return reduce_logical_impl<double>(op, A, rows, cols, dim, out, as_stream(s));
}

}  // extern "C"
