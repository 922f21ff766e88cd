// nt2cuda/tma.cuh -- bulk-copy (TMA) and mbarrier primitives for sm_103a.
//
// Streaming kernels stage their input tiles in shared memory with the Tensor
// Memory Accelerator: one thread issues a cp.async.bulk (1-D) or
// cp.async.bulk.tensor (2-D, through a tensor map) per tile, the copy
// completes on an mbarrier with an expected byte count, and the whole block
// waits on that barrier.  The copy engine keeps many tiles in flight without
// holding registers, which is what a latency-bound reduction needs.
//
// Every wait is bounded: mbar_wait gives up after a fixed number of
// try_wait rounds and reports failure, so a kernel can record an error and
// leave instead of spinning forever.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <mutex>

namespace nt2cuda {
namespace tma {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the barrier initialisation visible to the async (copy) proxy
__device__ __forceinline__ void fence_barrier_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier shared-memory accesses before later async-proxy writes
__device__ __forceinline__ void fence_proxy_async()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase)
{
  uint32_t ok;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait for the barrier's phase `phase` to complete.  Each try_wait
// round suspends for a hardware-defined time slice; kMaxRounds rounds bound
// the wait to well under a few seconds.
constexpr uint32_t kMaxRounds = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, uint32_t rounds = kMaxRounds)
{
  for (uint32_t i = 0; i < rounds; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

// 1-D bulk copy global -> shared (addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// 2-D tiled load through a tensor map; x is the innermost (contiguous)
// coordinate and must be a multiple of 16 bytes' worth of elements.
__device__ __forceinline__ void tensor_g2s_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 2-D tiled store shared -> global through a tensor map (a bulk group of
// this thread; complete it with bulk_commit and wait with bulk_wait*)
__device__ __forceinline__ void tensor_s2g_2d(const CUtensorMap* map, int x, int y, const void* src)
{
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map), "r"(x),
               "r"(y), "r"(smem_u32(src))
               : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// this thread's bulk groups but the N most recent have finished reading shared memory
template <int N> __device__ __forceinline__ void bulk_wait_read()
{
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// this thread's bulk groups but the N most recent have completed
template <int N> __device__ __forceinline__ void bulk_wait()
{
  asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}

// The CUDA driver API's cuTensorMapEncodeTiled, looked up once (null when
// the installed CUDA driver does not provide it).
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

}  // namespace tma
}  // namespace nt2cuda
