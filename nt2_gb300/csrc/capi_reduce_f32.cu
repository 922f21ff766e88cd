// capi_reduce_f32.cu -- C-ABI entry points of the FP32 reductions (reduce_impl.cuh).
#include "reduce_impl.cuh"

using namespace nt2cuda::detail_capi;

extern "C" {

nt2cuda_status nt2cuda_reduce_f32(int op, const float* A, size_t rows, size_t cols, int dim, float* out, int flags,
                                  nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  return reduce_impl<float>(op, A, rows, cols, dim, out, flags, as_stream(s));
}

nt2cuda_status nt2cuda_reduce_logical_f32(int op, const float* A, size_t rows, size_t cols, int dim, uint8_t* out,
                                          nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  return reduce_logical_impl<float>(op, A, rows, cols, dim, out, as_stream(s));
}

}  // extern "C"
