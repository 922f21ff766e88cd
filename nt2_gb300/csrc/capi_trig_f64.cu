// capi_trig_f64.cu -- nt2cuda_map_f64's trigonometric ops (double tables).
#include "trig_impl.cuh"

namespace nt2cuda {
namespace detail_capi {

nt2cuda_status map_trig(int op, const double* x, double* y, size_t n, bool fused, bool simd128, nt2cuda_stream s)
{
  return dispatch(op, x, y, n, fused, simd128, s);
}

}  // namespace detail_capi
}  // namespace nt2cuda
