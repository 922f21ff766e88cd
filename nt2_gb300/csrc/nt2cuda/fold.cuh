// nt2cuda/fold.cuh -- inner_fold (contiguous) and outer_fold (strided)
// reductions of an elementwise expression.
//
// NT2 maps sum/globalsum to inner_fold when the reduced dimension is the
// first non-singleton one and to outer_fold otherwise
// (modules/core/reduction/include/nt2/dsl/functions/reduction/run.hpp:30-104).
//   inner_fold: per outer slice, an N-lane accumulation over contiguous
//     elements, a horizontal sum and a scalar tail
//     (modules/core/reduction/include/nt2/core/functions/simd/inner_fold.hpp:49-66);
//     the OpenMP spawner splits long slices into blocks whose partials are
//     combined in arrival order (modules/arch/openmp/include/nt2/sdk/openmp/spawner/fold.hpp:49-66).
//   outer_fold: out[o][i] = fold over m of in[o][m][i], contiguous in i
//     (modules/core/reduction/include/nt2/core/functions/details/outer_fold_step.hpp:33-67).
// Here the element values come from an expression (so globalsum(X*Y) reads X
// and Y once, as NT2's fused fold_step does), FP32 accumulates with
// TwoSum-compensated partials when COMP is set, and the split of the work
// into warps and blocks depends only on the table's shape: partials are
// combined in index order, never in arrival order, so results are bitwise
// reproducible from run to run and across GPUs.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "expr.cuh"
#include "math.cuh"

namespace nt2cuda {
namespace fold {

// ------------------------------------------------ compensated accumulators
template <class T> struct acc { T s, c; };

template <bool COMP, class T> __device__ __forceinline__ void add(acc<T>& a, T x)
{
  using namespace math;
  if constexpr (COMP) {
    T t = nt2cuda::math::add(a.s, x);
    T z = sub(t, a.s);
    T e = nt2cuda::math::add(sub(a.s, sub(t, z)), sub(x, z));
    a.c = nt2cuda::math::add(a.c, e);
    a.s = t;
  } else {
    a.s = nt2cuda::math::add(a.s, x);
  }
}

template <bool COMP, class T> __device__ __forceinline__ acc<T> merge(acc<T> a, acc<T> b)
{
  using namespace math;
  if constexpr (COMP) {
    T t = nt2cuda::math::add(a.s, b.s);
    T z = sub(t, a.s);
    T e = nt2cuda::math::add(sub(a.s, sub(t, z)), sub(b.s, z));
    return acc<T>{t, nt2cuda::math::add(nt2cuda::math::add(a.c, b.c), e)};
  } else {
    return acc<T>{nt2cuda::math::add(a.s, b.s), T(0)};
  }
}

template <bool COMP, class T> __device__ __forceinline__ T result(acc<T> a)
{
  return COMP ? nt2cuda::math::add(a.s, a.c) : a.s;
}

// Butterfly over the warp; every lane ends with the same value.
template <bool COMP, class T> __device__ __forceinline__ acc<T> warp_merge(acc<T> a)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    acc<T> o;
    o.s = __shfl_xor_sync(0xffffffffu, a.s, off);
    o.c = __shfl_xor_sync(0xffffffffu, a.c, off);
    // combine in lane order so every lane computes the same value
    a = ((threadIdx.x & 31) & off) ? merge<COMP>(o, a) : merge<COMP>(a, o);
  }
  return a;
}

// ------------------------------------------------------------ inner fold
// Work unit: one warp reduces the segment [r0, r1) of column j, where the
// column is split into `splits` segments of `seg` elements (seg a multiple
// of 32*V).  With splits > 1 the warp writes its partial to scratch and the
// last warp of the column combines the column's partials in segment order.
struct inner_shape {
  size_t rows, cols, seg, splits;
};

template <bool COMP, int V, int U, class T, class E>
__global__ void __launch_bounds__(256) k_inner(E e, inner_shape sh, T* __restrict__ out,
                                               acc<T>* __restrict__ partials, unsigned* __restrict__ counters)
{
  const int lane = threadIdx.x & 31;
  const size_t warps_total = (size_t)gridDim.x * (blockDim.x >> 5);
  const size_t units = sh.cols * sh.splits;
  for (size_t w = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < units; w += warps_total) {
    const size_t j = w / sh.splits, sp = w % sh.splits;
    const size_t r0 = sp * sh.seg;
    const size_t r1 = (r0 + sh.seg < sh.rows) ? r0 + sh.seg : sh.rows;
    const size_t base = j * sh.rows;
    acc<T> a[V];
#pragma unroll
    for (int l = 0; l < V; ++l) a[l] = acc<T>{T(0), T(0)};
    // full V-groups
    const size_t g0 = r0 / V, g1 = r1 / V;   // r0 is a multiple of V
    size_t g = g0 + lane;
    for (; g + (size_t)(U - 1) * 32 < g1; g += (size_t)U * 32) {
      regs<E, V> rr[U];
#pragma unroll
      for (int u = 0; u < U; ++u) rr[u].template load<true>(e, base + (g + (size_t)u * 32) * V);
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int l = 0; l < V; ++l) add<COMP>(a[l], (T)rr[u].template get<false>(e, l));
    }
    for (; g < g1; g += 32) {
      regs<E, V> rr;
      rr.template load<true>(e, base + g * V);
#pragma unroll
      for (int l = 0; l < V; ++l) add<COMP>(a[l], (T)rr.template get<false>(e, l));
    }
    // ragged end of the segment (only when rows % V != 0 or V == 1)
    for (size_t r = g1 * V + lane; r < r1; r += 32) {
      regs<E, 1> rr;
      rr.template load<false>(e, base + r);
      add<COMP>(a[0], (T)rr.template get<false>(e, 0));
    }
    acc<T> t = a[0];
#pragma unroll
    for (int l = 1; l < V; ++l) t = merge<COMP>(t, a[l]);
    t = warp_merge<COMP>(t);
    if (sh.splits == 1) {
      if (lane == 0) out[j] = result<COMP>(t);
      continue;
    }
    unsigned last = 0;
    if (lane == 0) {
      partials[w] = t;
      __threadfence();
      unsigned prev = atomicAdd(&counters[j], 1u);
      last = (prev == (unsigned)sh.splits - 1u);
      if (last) counters[j] = 0u;   // ready for the next call on this scratch
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) continue;
    __threadfence();
    // combine the column's partials in segment order: lane k folds
    // segments k, k+32, ... then the butterfly merges lanes in order
    acc<T> c{T(0), T(0)};
    for (size_t q = lane; q < sh.splits; q += 32) {
      const acc<T>* p = partials + j * sh.splits + q;
      acc<T> v{__ldcg(&p->s), __ldcg(&p->c)};
      c = merge<COMP>(c, v);
    }
    c = warp_merge<COMP>(c);
    if (lane == 0) out[j] = result<COMP>(c);
  }
}

// Short columns (rows < 32): one thread folds one whole column.
template <bool COMP, class T, class E>
__global__ void __launch_bounds__(256) k_inner_short(E e, size_t rows, size_t cols, T* __restrict__ out)
{
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < cols; j += (size_t)gridDim.x * blockDim.x) {
    acc<T> a{T(0), T(0)};
    for (size_t r = 0; r < rows; ++r) {
      regs<E, 1> rr;
      rr.template load<false>(e, j * rows + r);
      add<COMP>(a, (T)rr.template get<false>(e, 0));
    }
    out[j] = result<COMP>(a);
  }
}

// ------------------------------------------------------------ outer fold
// Row sums of a rows x cols column-major table.  A block owns a strip of
// 32*V rows (one V-group per lane) and a chunk of `cchunk` columns; its 8
// warps take the chunk's columns round-robin, and the block merges the
// warps' partials in warp order.  With splits > 1 the block's per-row
// partials go to scratch and the last block of the strip merges them in
// chunk order.
struct outer_shape {
  size_t rows, cols, cchunk, splits, strips;
};

template <bool COMP, int V, int U, class T, class E>
__global__ void __launch_bounds__(256) k_outer(E e, outer_shape sh, T* __restrict__ out,
                                               acc<T>* __restrict__ partials, unsigned* __restrict__ counters)
{
  constexpr int STRIP = 32 * V;
  __shared__ acc<T> red[8][STRIP];
  __shared__ unsigned is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t units = sh.strips * sh.splits;
  for (size_t b = blockIdx.x; b < units; b += gridDim.x) {
    const size_t strip = b / sh.splits, sp = b % sh.splits;
    const size_t row0 = strip * STRIP + (size_t)lane * V;   // first row of this lane
    const size_t m0 = sp * sh.cchunk;
    const size_t m1 = (m0 + sh.cchunk < sh.cols) ? m0 + sh.cchunk : sh.cols;
    const bool full = row0 + V <= sh.rows;
    acc<T> a[V];
#pragma unroll
    for (int l = 0; l < V; ++l) a[l] = acc<T>{T(0), T(0)};
    if (full) {
      size_t m = m0 + warp;
      for (; m + (size_t)(U - 1) * 8 < m1; m += (size_t)U * 8) {
        regs<E, V> rr[U];
#pragma unroll
        for (int u = 0; u < U; ++u) rr[u].template load<true>(e, (m + (size_t)u * 8) * sh.rows + row0);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int l = 0; l < V; ++l) add<COMP>(a[l], (T)rr[u].template get<false>(e, l));
      }
      for (; m < m1; m += 8) {
        regs<E, V> rr;
        rr.template load<true>(e, m * sh.rows + row0);
#pragma unroll
        for (int l = 0; l < V; ++l) add<COMP>(a[l], (T)rr.template get<false>(e, l));
      }
    } else if (row0 < sh.rows) {
      for (size_t m = m0 + warp; m < m1; m += 8)
#pragma unroll
        for (int l = 0; l < V; ++l)
          if (row0 + l < sh.rows) {
            regs<E, 1> rr;
            rr.template load<false>(e, m * sh.rows + row0 + l);
            add<COMP>(a[l], (T)rr.template get<false>(e, 0));
          }
    }
#pragma unroll
    for (int l = 0; l < V; ++l) red[warp][lane * V + l] = a[l];
    __syncthreads();
    // thread t < STRIP merges row t of the strip over the 8 warps in order
    acc<T> rsum{T(0), T(0)};
    const size_t row = strip * STRIP + threadIdx.x;
    if (threadIdx.x < STRIP) {
      rsum = red[0][threadIdx.x];
#pragma unroll
      for (int w = 1; w < 8; ++w) rsum = merge<COMP>(rsum, red[w][threadIdx.x]);
    }
    if (sh.splits == 1) {
      if (threadIdx.x < STRIP && row < sh.rows) out[row] = result<COMP>(rsum);
      __syncthreads();
      continue;
    }
    if (threadIdx.x < STRIP) partials[b * STRIP + threadIdx.x] = rsum;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned prev = atomicAdd(&counters[strip], 1u);
      is_last = (prev == (unsigned)sh.splits - 1u);
      if (is_last) counters[strip] = 0u;
    }
    __syncthreads();
    if (is_last) {
      __threadfence();
      if (threadIdx.x < STRIP && row < sh.rows) {
        acc<T> c{T(0), T(0)};
        size_t q = 0;
        for (; q + 8 <= sh.splits; q += 8) {
          acc<T> v[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const acc<T>* p = partials + (strip * sh.splits + q + k) * STRIP + threadIdx.x;
            v[k] = acc<T>{__ldcg(&p->s), __ldcg(&p->c)};
          }
#pragma unroll
          for (int k = 0; k < 8; ++k) c = merge<COMP>(c, v[k]);
        }
        for (; q < sh.splits; ++q) {
          const acc<T>* p = partials + (strip * sh.splits + q) * STRIP + threadIdx.x;
          c = merge<COMP>(c, acc<T>{__ldcg(&p->s), __ldcg(&p->c)});
        }
        out[row] = result<COMP>(c);
      }
    }
    __syncthreads();
  }
}

}  // namespace fold
}  // namespace nt2cuda
