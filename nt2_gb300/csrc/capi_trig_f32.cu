// capi_trig_f32.cu -- nt2cuda_map_f32's trigonometric ops, nt2cuda_atan2_f32 and nt2cuda_pow_f32 (float tables).
#include "trig_impl.cuh"

namespace nt2cuda {
namespace detail_capi {

nt2cuda_status map_trig(int op, const float* x, float* y, size_t n, bool fused, bool simd128, nt2cuda_stream s)
{
  return dispatch(op, x, y, n, fused, simd128, s);
}

}  // namespace detail_capi
}  // namespace nt2cuda

extern "C" nt2cuda_status nt2cuda_atan2_f32(const float* a0, const float* a1, float* out, size_t n, int flags,
                                             nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!a0 || !a1 || !out)) return NT2CUDA_ERR_ARG;
  if (flags & ~NT2CUDA_MAP_FUSED) return NT2CUDA_ERR_ARG;
  return nt2cuda::detail_capi::binary_impl<nt2cuda::tag::atan2_>(a0, a1, out, n, (flags & NT2CUDA_MAP_FUSED) != 0, s);
}

extern "C" nt2cuda_status nt2cuda_pow_f32(const float* a0, const float* a1, float* out, size_t n, int flags,
                                           nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!a0 || !a1 || !out)) return NT2CUDA_ERR_ARG;
  if (flags & ~NT2CUDA_MAP_FUSED) return NT2CUDA_ERR_ARG;
  return nt2cuda::detail_capi::binary_impl<nt2cuda::tag::pow_>(a0, a1, out, n, (flags & NT2CUDA_MAP_FUSED) != 0, s);
}
