// nt2cuda/memory.cuh -- 16-byte global loads and stores for streaming tables.
//
// Tables on the evaluator's path are read once and written once per
// evaluation, so inputs are read through the non-coherent path without L1
// allocation and outputs are stored with the evict-first (.cs) policy.  An
// input may be the same table as an output of its statement (Y = a*X + Y):
// every element is then read, before it is written, by the one thread that
// writes it, and never read again, so no stale line can be observed.
// ld_plain is the coherent load used for single elements.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nt2cuda {
namespace mem {

template <int NB> struct chunk;  // raw storage of NB bytes
template <> struct chunk<16> { uint4 v; };
template <> struct chunk<8> { uint2 v; };
template <> struct chunk<4> { uint32_t v; };
template <> struct chunk<2> { uint16_t v; };
template <> struct chunk<1> { uint8_t v; };

// Streaming, read-only load of NB bytes (NB-aligned address).
template <int NB> __device__ __forceinline__ chunk<NB> ld_stream(const void* p);
template <> __device__ __forceinline__ chunk<16> ld_stream<16>(const void* p)
{
  chunk<16> c;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(c.v.x), "=r"(c.v.y), "=r"(c.v.z), "=r"(c.v.w) : "l"(p));
  return c;
}
template <> __device__ __forceinline__ chunk<8> ld_stream<8>(const void* p)
{
  chunk<8> c;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0,%1}, [%2];" : "=r"(c.v.x), "=r"(c.v.y) : "l"(p));
  return c;
}
template <> __device__ __forceinline__ chunk<4> ld_stream<4>(const void* p)
{
  chunk<4> c;
  asm volatile("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(c.v) : "l"(p));
  return c;
}
template <> __device__ __forceinline__ chunk<2> ld_stream<2>(const void* p)
{
  chunk<2> c;
  c.v = __ldg(reinterpret_cast<const unsigned short*>(p));
  return c;
}
template <> __device__ __forceinline__ chunk<1> ld_stream<1>(const void* p)
{
  chunk<1> c;
  c.v = __ldg(reinterpret_cast<const unsigned char*>(p));
  return c;
}

// Coherent load (the address may have been written earlier by this thread);
// the memory clobber keeps it after those stores.
template <int NB> __device__ __forceinline__ chunk<NB> ld_plain(const void* p);
template <> __device__ __forceinline__ chunk<16> ld_plain<16>(const void* p)
{
  chunk<16> c;
  asm volatile("ld.global.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(c.v.x), "=r"(c.v.y), "=r"(c.v.z), "=r"(c.v.w) : "l"(p) : "memory");
  return c;
}
template <> __device__ __forceinline__ chunk<8> ld_plain<8>(const void* p)
{
  chunk<8> c;
  asm volatile("ld.global.v2.u32 {%0,%1}, [%2];" : "=r"(c.v.x), "=r"(c.v.y) : "l"(p) : "memory");
  return c;
}
template <> __device__ __forceinline__ chunk<4> ld_plain<4>(const void* p)
{
  chunk<4> c;
  asm volatile("ld.global.u32 %0, [%1];" : "=r"(c.v) : "l"(p) : "memory");
  return c;
}
template <> __device__ __forceinline__ chunk<2> ld_plain<2>(const void* p)
{
  chunk<2> c;
  unsigned short v;
  asm volatile("ld.global.u16 %0, [%1];" : "=h"(v) : "l"(p) : "memory");
  c.v = v;
  return c;
}
template <> __device__ __forceinline__ chunk<1> ld_plain<1>(const void* p)
{
  chunk<1> c;
  unsigned short v;
  asm volatile("ld.global.u8 %0, [%1];" : "=h"(v) : "l"(p) : "memory");
  c.v = (uint8_t)v;
  return c;
}

// Evict-first store of NB bytes.
template <int NB> __device__ __forceinline__ void st_stream(void* p, chunk<NB> c);
template <> __device__ __forceinline__ void st_stream<16>(void* p, chunk<16> c)
{
  asm volatile("st.global.cs.v4.u32 [%0], {%1,%2,%3,%4};"
               :: "l"(p), "r"(c.v.x), "r"(c.v.y), "r"(c.v.z), "r"(c.v.w) : "memory");
}
template <> __device__ __forceinline__ void st_stream<8>(void* p, chunk<8> c)
{
  asm volatile("st.global.cs.v2.u32 [%0], {%1,%2};" :: "l"(p), "r"(c.v.x), "r"(c.v.y) : "memory");
}
template <> __device__ __forceinline__ void st_stream<4>(void* p, chunk<4> c)
{
  asm volatile("st.global.cs.u32 [%0], %1;" :: "l"(p), "r"(c.v) : "memory");
}
template <> __device__ __forceinline__ void st_stream<2>(void* p, chunk<2> c)
{
  unsigned short v = c.v;
  asm volatile("st.global.cs.u16 [%0], %1;" :: "l"(p), "h"(v) : "memory");
}
template <> __device__ __forceinline__ void st_stream<1>(void* p, chunk<1> c)
{
  unsigned short v = c.v;
  asm volatile("st.global.cs.u8 [%0], %1;" :: "l"(p), "h"(v) : "memory");
}

// Load V contiguous elements of T starting at element i (the address of
// element i is aligned to min(16, V*sizeof(T)) bytes).
template <class T, int V, bool Stream>
__device__ __forceinline__ void load_vec(const T* base, size_t i, T (&out)[V])
{
  constexpr int BYTES = V * (int)sizeof(T);
  constexpr int NB = BYTES >= 16 ? 16 : BYTES;
  constexpr int NC = BYTES / NB;
  const char* p = reinterpret_cast<const char*>(base + i);
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    chunk<NB> ch = Stream ? ld_stream<NB>(p + c * NB) : ld_plain<NB>(p + c * NB);
    memcpy(reinterpret_cast<char*>(out) + c * NB, &ch, NB);
  }
}

template <class T, int V>
__device__ __forceinline__ void store_vec(T* base, size_t i, const T (&in)[V])
{
  constexpr int BYTES = V * (int)sizeof(T);
  constexpr int NB = BYTES >= 16 ? 16 : BYTES;
  constexpr int NC = BYTES / NB;
  char* p = reinterpret_cast<char*>(base + i);
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    chunk<NB> ch;
    memcpy(&ch, reinterpret_cast<const char*>(in) + c * NB, NB);
    st_stream<NB>(p + c * NB, ch);
  }
}

// Ask the L2 for the 128-byte line holding p (no register result, no fault
// path taken by the kernels: they only prefetch addresses they load).  It may
// be issued before pdl_begin() for data the previous grid writes: the L2 is
// the GPU's point of coherence for device memory, so a line fetched early is
// updated by that grid's stores, and the loads after the wait see them.
__device__ __forceinline__ void prefetch_l2(const void* p)
{
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Kernels launched as programmatic dependents (launch.cuh) begin here: wait
// until the previous grid on the stream has completed and its writes are
// visible, then let the next grid be scheduled.
__device__ __forceinline__ void pdl_begin()
{
  asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace mem
}  // namespace nt2cuda
