// internal.cuh -- helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <mutex>
#include <unordered_map>
#include "../../include/nt2cuda.h"

namespace nt2cuda {
namespace detail_capi {

inline cudaStream_t as_stream(nt2cuda_stream s) { return reinterpret_cast<cudaStream_t>(s); }

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

// Per-stream scratch for the multi-block folds.  Each stream gets its own
// buffer so folds enqueued on different streams never share partials;
// calls on one stream are ordered, so they can reuse it.  The buffer only
// grows; growing synchronises the stream first.
struct scratch_pool {
  struct entry { void* p = nullptr; size_t bytes = 0; };
  std::mutex m;
  std::unordered_map<uintptr_t, entry> by_stream;
};
inline scratch_pool& pool() { static scratch_pool p; return p; }

// slot 0: fold partials and counters; slot 1: batched-launch descriptors.
inline nt2cuda_status stream_scratch(cudaStream_t s, size_t bytes, void** out, int slot = 0)
{
  int dev = 0;
  cudaGetDevice(&dev);
  uintptr_t key = (reinterpret_cast<uintptr_t>(s) * 64u + (uintptr_t)dev) * 4u + (uintptr_t)slot;
  scratch_pool& P = pool();
  std::lock_guard<std::mutex> g(P.m);
  scratch_pool::entry& e = P.by_stream[key];
  if (e.bytes < bytes) {
    if (e.p) {
      cudaStreamSynchronize(s);
      cudaFree(e.p);
      e.p = nullptr;
      e.bytes = 0;
    }
    size_t want = bytes < 4096 ? 4096 : bytes;
    cudaError_t err = cudaMalloc(&e.p, want);
    if (err != cudaSuccess) { e.p = nullptr; return from_cuda(err); }
    // counters at the front of the scratch start (and are left) at zero
    err = cudaMemsetAsync(e.p, 0, want, s);
    if (err != cudaSuccess) return from_cuda(err);
    e.bytes = want;
  }
  *out = e.p;
  return NT2CUDA_OK;
}

}  // namespace detail_capi
}  // namespace nt2cuda
