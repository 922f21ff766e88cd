// internal.cuh -- helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <mutex>
#include <unordered_map>
#include <nvtx3/nvToolsExt.h>
#include "../../include/nt2cuda.h"
#include "nt2cuda/scratch.cuh"

namespace nt2cuda {
namespace detail_capi {

inline cudaStream_t as_stream(nt2cuda_stream s) { return reinterpret_cast<cudaStream_t>(s); }

// An NVTX range named after the C-ABI entry point around its body, so that
// Nsight tools attribute the launches to the call (no cost without a tool).
struct nvtx_range {
  explicit nvtx_range(const char* name) { nvtxRangePushA(name); }
  ~nvtx_range() { nvtxRangePop(); }
  nvtx_range(const nvtx_range&) = delete;
  nvtx_range& operator=(const nvtx_range&) = delete;
};
#define NT2CUDA_NVTX_RANGE ::nt2cuda::detail_capi::nvtx_range nt2cuda_nvtx_range_(__func__)

// Remember the last CUDA error code seen by an entry point.
inline int& last_cuda_error() { static thread_local int e = 0; return e; }

inline nt2cuda_status from_cuda(cudaError_t e, nt2cuda_status on_error = NT2CUDA_ERR_CUDA)
{
  if (e == cudaSuccess) return NT2CUDA_OK;
  last_cuda_error() = (int)e;
  if (e == cudaErrorMemoryAllocation) return NT2CUDA_ERR_OOM;
  if (e == cudaErrorInvalidValue) return NT2CUDA_ERR_ARG;
  return on_error;
}

inline nt2cuda_status launch_status(cudaError_t e)
{
  if (e == cudaErrorInvalidValue) { last_cuda_error() = (int)e; return NT2CUDA_ERR_ALIAS; }
  if (e != cudaSuccess) return from_cuda(e, NT2CUDA_ERR_LAUNCH);
  e = cudaGetLastError();
  return from_cuda(e, NT2CUDA_ERR_LAUNCH);
}

inline nt2cuda_status stream_scratch(cudaStream_t s, size_t bytes, void** out, int slot = 0)
{
  return from_cuda(nt2cuda::stream_scratch(s, bytes, out, slot));
}

// Load the single-request FP32 Black-Scholes kernels of one (cdf, precision)
// pair ahead of their first launch (capi_transform.cu).
void warm_blackscholes_f32(int cdf_kind, int precision);

// y = op(x) for the trigonometric ops of nt2cuda_map_*, reduced element by
// element or (simd128) over 16-byte packs (capi_trig.cu, a translation unit of
// its own so that the build compiles it in parallel).
nt2cuda_status map_trig(int op, const float* x, float* y, size_t n, bool fused, bool simd128, nt2cuda_stream s);
nt2cuda_status map_trig(int op, const double* x, double* y, size_t n, bool fused, bool simd128, nt2cuda_stream s);
// capi_trigx_f32.cu / capi_trigx_f64.cu: ops NT2CUDA_OP_CSC..NT2CUDA_OP_SINCPI
nt2cuda_status map_trigx(int op, const float* x, float* y, size_t n, bool fused, bool simd128, nt2cuda_stream s);
nt2cuda_status map_trigx(int op, const double* x, double* y, size_t n, bool fused, bool simd128, nt2cuda_stream s);
// capi_trigx_fwd{,128}_f32.cu / _f64.cu: the reduced ops of map_trigx in NT2's scalar / 128-bit form
nt2cuda_status trigx_fwd_scalar(int op, const float* x, float* y, size_t n, bool fused, nt2cuda_stream s);
nt2cuda_status trigx_fwd_scalar(int op, const double* x, double* y, size_t n, bool fused, nt2cuda_stream s);
nt2cuda_status trigx_fwd_simd128(int op, const float* x, float* y, size_t n, bool fused, nt2cuda_stream s);
nt2cuda_status trigx_fwd_simd128(int op, const double* x, double* y, size_t n, bool fused, nt2cuda_stream s);
// capi_expfam_f32.cu / capi_expfam_f64.cu: ops NT2CUDA_OP_CBRT..NT2CUDA_OP_REALLOG, NT2CUDA_OP_ATANH..SINHC
nt2cuda_status map_expfam(int op, const float* x, float* y, size_t n, bool fused, nt2cuda_stream s);
nt2cuda_status map_expfam(int op, const double* x, double* y, size_t n, bool fused, nt2cuda_stream s);

}  // namespace detail_capi
}  // namespace nt2cuda
