// capi_trigx_f32.cu -- nt2cuda_map_f32's composed trigonometric ops and nt2cuda_sincos_f32 (float tables).
#include "trigx_impl.cuh"

namespace nt2cuda {
namespace detail_capi {

nt2cuda_status map_trigx(int op, const float* x, float* y, size_t n, bool fused, bool simd128, nt2cuda_stream s)
{
  return trigx_dispatch(op, x, y, n, fused, simd128, s);
}

}  // namespace detail_capi
}  // namespace nt2cuda

extern "C" nt2cuda_status nt2cuda_sincos_f32(int form, const float* x, float* s, float* c, size_t n, int flags,
                                             nt2cuda_stream stream)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!x || !s || !c)) return NT2CUDA_ERR_ARG;
  if (flags & ~(NT2CUDA_MAP_FUSED | NT2CUDA_MAP_SIMD128)) return NT2CUDA_ERR_ARG;
  if (form < NT2CUDA_SINCOS || form > NT2CUDA_SINHCOSH) return NT2CUDA_ERR_ARG;
  if (n == 0) return NT2CUDA_OK;
  return nt2cuda::detail_capi::sincos_dispatch(form, x, s, c, n, (flags & NT2CUDA_MAP_FUSED) != 0,
                                               (flags & NT2CUDA_MAP_SIMD128) != 0, stream);
}
