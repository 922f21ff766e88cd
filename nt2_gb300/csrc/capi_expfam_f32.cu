// capi_expfam_f32.cu -- nt2cuda_map_f32's exponential-family ops and nt2cuda_map2_f32 (float tables).
#include "expfam_impl.cuh"

namespace nt2cuda {
namespace detail_capi {

nt2cuda_status map_expfam(int op, const float* x, float* y, size_t n, bool fused, nt2cuda_stream s)
{
  return fused ? expfam_impl<true>(op, x, y, n, s) : expfam_impl<false>(op, x, y, n, s);
}

}  // namespace detail_capi
}  // namespace nt2cuda

extern "C" nt2cuda_status nt2cuda_map2_f32(int op, const float* a0, const float* a1, float* out, size_t n, int flags,
                                           nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!a0 || !a1 || !out)) return NT2CUDA_ERR_ARG;
  if (flags & ~NT2CUDA_MAP_FUSED) return NT2CUDA_ERR_ARG;
  // atan2 and pow (and realpow, its alias) are built with the trigonometric ops
  if (op == NT2CUDA_OP2_ATAN2) return nt2cuda_atan2_f32(a0, a1, out, n, flags, s);
  if (op == NT2CUDA_OP2_POW || op == NT2CUDA_OP2_REALPOW) return nt2cuda_pow_f32(a0, a1, out, n, flags, s);
  const bool fused = (flags & NT2CUDA_MAP_FUSED) != 0;
  return fused ? nt2cuda::detail_capi::map2_impl<true>(op, a0, a1, out, n, s)
               : nt2cuda::detail_capi::map2_impl<false>(op, a0, a1, out, n, s);
}
