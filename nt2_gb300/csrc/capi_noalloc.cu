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
//
// The result is within the error bound of nt2cuda_dot_f32 and bitwise
// reproducible from one call of this entry point to the next, but not bit
// for bit nt2cuda_dot_f32's: that entry point takes the TMA fold for long
// aligned vectors, this one always takes the register-staged fold kernel.
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
struct scratch_slot {
  unsigned long long ctx_id = 0;     // the context the address belongs to (0: none yet)
  void* addr = nullptr;
};
scratch_slot g_scratch[kMaxDevices];

// The CUDA driver API's identifier of the current context: unique over the process,
// so a context torn down (cudaDeviceReset) and created again gets a new one.
using ctx_get_current_fn = int (*)(void**);
using ctx_get_id_fn = int (*)(void*, unsigned long long*);
cudaError_t current_context_id(unsigned long long* id)
{
  static ctx_get_current_fn get_current = nullptr;
  static ctx_get_id_fn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<ctx_get_current_fn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<ctx_get_id_fn>(p);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return cudaErrorNotSupported;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0) return cudaErrorDeviceUninitialized;
  if (!ctx) {                                  // no context yet: 0, which no context has
    *id = 0;
    return cudaSuccess;
  }
  return get_id(ctx, id) == 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

// Once per device and context, with that device current: look up the device
// address of the scratch array.  Done by the first call on each device, and
// again by the first call after the device's context was reset.
nt2cuda_status scratch_address(void** out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return from_cuda(e);
  if (dev < 0 || dev >= kMaxDevices) return NT2CUDA_ERR_ARG;
  unsigned long long ctx = 0;
  if ((e = current_context_id(&ctx)) != cudaSuccess) return from_cuda(e);
  std::lock_guard<std::mutex> g(g_setup_mutex);
  scratch_slot& slot = g_scratch[dev];
  if (ctx == 0 || slot.ctx_id != ctx || !slot.addr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);    // also creates the context when there is none
    if (e != cudaSuccess) return from_cuda(e);
    if ((e = current_context_id(&ctx)) != cudaSuccess) return from_cuda(e);
    slot.addr = p;
    slot.ctx_id = ctx;
  }
  *out = slot.addr;
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
