// nt2cuda/scratch.cuh -- per-stream device scratch for multi-block kernels.
//
// The folds keep per-block partials and arrival counters in global memory.
// Each (stream, device, slot) gets its own buffer, so kernels enqueued on
// different streams never share scratch; calls on one stream are ordered and
// reuse it.  A buffer only grows; growing synchronises its stream first.  The
// first call on a stream allocates (cudaMalloc), so make it before capturing
// that stream into a CUDA graph.  The folds' arrival counters have a slot of
// their own: they start at zero (a buffer is cleared when allocated), every
// fold leaves the ones it used at zero, and nothing else is written there --
// partials, which other kernels overwrite freely, live in another slot.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include <unordered_map>

namespace nt2cuda {

struct scratch_pool {
  struct entry { void* p = nullptr; size_t bytes = 0; };
  std::mutex m;
  std::unordered_map<uintptr_t, entry> by_key;
  unsigned long long allocations = 0;     // cudaMalloc calls made for scratch so far
};
inline scratch_pool& global_scratch_pool() { static scratch_pool p; return p; }

// slot 0: fold arrival counters only; slot 1: per-call data (batched-launch
// descriptors, scan flags and carries); slot 2: fold partials; slot 3
// (kResultSlot): device results the C++ front end reads back (globalsum).
constexpr int kResultSlot = 3;
inline cudaError_t stream_scratch(cudaStream_t s, size_t bytes, void** out, int slot = 0);

// The two buffers of a fold: ncounters zero-valued arrival counters and room
// for npartials partial states of `partial_bytes` each.
inline cudaError_t fold_scratch(cudaStream_t s, size_t ncounters, size_t npartials, size_t partial_bytes,
                                unsigned** counters, void** partials)
{
  void* c = nullptr;
  cudaError_t e = stream_scratch(s, ncounters * sizeof(unsigned), &c, 0);
  if (e != cudaSuccess) return e;
  e = stream_scratch(s, npartials * partial_bytes, partials, 2);
  *counters = (unsigned*)c;
  return e;
}

inline cudaError_t stream_scratch(cudaStream_t s, size_t bytes, void** out, int slot)
{
  int dev = 0;
  cudaGetDevice(&dev);
  uintptr_t key = (reinterpret_cast<uintptr_t>(s) * 64u + (uintptr_t)dev) * 4u + (uintptr_t)slot;
  scratch_pool& P = global_scratch_pool();
  std::lock_guard<std::mutex> g(P.m);
  scratch_pool::entry& e = P.by_key[key];
  if (e.bytes < bytes) {
    if (e.p) {
      cudaStreamSynchronize(s);
      cudaFree(e.p);
      e.p = nullptr;
      e.bytes = 0;
    }
    size_t want = bytes < 4096 ? 4096 : bytes;
    cudaError_t err = cudaMalloc(&e.p, want);
    if (err != cudaSuccess) { e.p = nullptr; return err; }
    ++P.allocations;
    err = cudaMemsetAsync(e.p, 0, want, s);
    if (err != cudaSuccess) return err;
    e.bytes = want;
  }
  *out = e.p;
  return cudaSuccess;
}

}  // namespace nt2cuda
