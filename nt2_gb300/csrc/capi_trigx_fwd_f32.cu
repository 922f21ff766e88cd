// capi_trigx_fwd_f32.cu -- the reduced composed trigonometric ops of nt2cuda_map_f32 in
// NT2's scalar form (float tables).
#include "trigx_impl.cuh"

namespace nt2cuda {
namespace detail_capi {

nt2cuda_status trigx_fwd_scalar(int op, const float* x, float* y, size_t n, bool fused, nt2cuda_stream s)
{
  return fused ? recip_impl<true, false>(op, x, y, n, s) : recip_impl<false, false>(op, x, y, n, s);
}

}  // namespace detail_capi
}  // namespace nt2cuda
