// capi_trigx_f64.cu -- nt2cuda_map_f64's composed trigonometric ops (double tables).
#include "trigx_impl.cuh"

namespace nt2cuda {
namespace detail_capi {

nt2cuda_status map_trigx(int op, const double* x, double* y, size_t n, bool fused, bool simd128, nt2cuda_stream s)
{
  return trigx_dispatch(op, x, y, n, fused, simd128, s);
}

}  // namespace detail_capi
}  // namespace nt2cuda
