// capi_noalloc.cu -- globalsum(X*Y) (the sdot fold) without any allocation.
//
// Some callers cannot call cudaMalloc: a host whose device memory is handed
// out by another allocator (a framework's caching pool that owns the GPU's
// memory and does not expect outside allocations), or a latency-bound loop
// where cudaMalloc's device-wide synchronisation and unpredictable cost are
// not acceptable.  nt2cuda_dot_f32 allocates its per-stream scratch on first
// use, so it is closed to them.  nt2cuda_dot_f32_noalloc runs the same fold
// kernel with its scratch in a fixed array in device memory, defined below,
// that exists for as long as the library is loaded on every GPU that loads it.
//
// The array holds one arrival counter and one partial sum per 16384-element
// segment, so n is limited to NT2CUDA_DOT_NOALLOC_MAX_N (2^30) elements and
// the array is 256 B + 64 Ki partials x 8 B = 512.25 KiB.  All calls share
// it: two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on it; calls on one stream are ordered and
// safe.  The counter is cleared by a memset before every launch, so a call
// does not depend on what an earlier call left behind.
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/fold.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;
using nt2cuda::fold::acc;

namespace {

constexpr size_t kSeg = (size_t)32 * 4 * 128;                         // a warp's segment, as nt2cuda_dot_f32
constexpr size_t kMaxSplits = (size_t)NT2CUDA_DOT_NOALLOC_MAX_N / kSeg;
constexpr size_t kCounterBytes = 256;
constexpr size_t kScratchBytes = kCounterBytes + kMaxSplits * sizeof(acc<float>);

// The fixed scratch.  In host code this name is only a handle for
// cudaGetSymbolAddress, never a device address.
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: look up the device address of
// the scratch array.  Done by the first call on each device.
nt2cuda_status scratch_address(void** out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return from_cuda(e);
  if (dev < 0 || dev >= kMaxDevices) return NT2CUDA_ERR_ARG;
  std::lock_guard<std::mutex> g(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return from_cuda(e);
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return NT2CUDA_OK;
}

template <bool COMP>
nt2cuda_status dot_noalloc(const float* x, const float* y, size_t n, float* out, cudaStream_t s)
{
  using E = node<tag::multiplies_, term<float>, term<float>>;
  E e{term<float>{x}, term<float>{y}};
  if (n < 32) {
    size_t rows = n, cols = 1;
    float* o = out;
    void* args[] = {&e, &rows, &cols, &o};
    return launch_status(launch_persistent(fold::k_inner_short<fold::op_sum<COMP>, float, E>, 1, 256, 1, s, args));
  }
  void* base = nullptr;
  nt2cuda_status st = scratch_address(&base);
  if (st != NT2CUDA_OK) return st;
  unsigned* counters = (unsigned*)base;
  acc<float>* partials = (acc<float>*)((char*)base + kCounterBytes);
  cudaError_t ce = cudaMemsetAsync(counters, 0, sizeof(unsigned), s);
  if (ce != cudaSuccess) return from_cuda(ce);
  fold::inner_shape sh;
  sh.rows = n;
  sh.cols = 1;
  sh.seg = kSeg;
  sh.splits = (n + kSeg - 1) / kSeg;
  const bool vec = ((((uintptr_t)x | (uintptr_t)y) & 15u) == 0) && (n % 4 == 0);
  float* o = out;
  void* args[] = {&e, &sh, &o, &partials, &counters};
  const size_t threads = sh.splits * 32;
  if (vec) return launch_status(launch_persistent(fold::k_inner<fold::op_sum<COMP>, 4, 4, float, E>, threads, 256, 4, s, args));
  return launch_status(launch_persistent(fold::k_inner<fold::op_sum<COMP>, 1, 4, float, E>, threads, 256, 4, s, args));
}

}  // namespace

extern "C" nt2cuda_status nt2cuda_dot_f32_noalloc(const float* x, const float* y, size_t n, float* out,
                                                  int compensated, nt2cuda_stream stream)
{
  if ((n && (!x || !y)) || !out) return NT2CUDA_ERR_ARG;
  if (n > (size_t)NT2CUDA_DOT_NOALLOC_MAX_N) return NT2CUDA_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (n == 0) return from_cuda(cudaMemsetAsync(out, 0, sizeof(float), s));
  return compensated ? dot_noalloc<true>(x, y, n, out, s) : dot_noalloc<false>(x, y, n, out, s);
}
