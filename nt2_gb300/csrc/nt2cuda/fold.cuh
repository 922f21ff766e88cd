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

// The value of a compensated pair.  Once the running sum is not finite (an
// overflow, an infinite or NaN term) its compensation is NaN and the sum
// itself is the result, as in NT2's plain float sum: inf stays inf.
template <bool COMP, class T> __device__ __forceinline__ T result(acc<T> a)
{
  if constexpr (COMP) {
    const T r = nt2cuda::math::add(a.s, a.c);
    return r != r ? a.s : r;
  } else {
    return a.s;
  }
}

// ------------------------------------------------------------ operations
// A reduction is NT2's reduction_<Tag, Bop, Neutral>
// (boost/simd/reduction/functions/sum.hpp:26-29, maximum.hpp:30, minimum.hpp:29,
// prod.hpp:26, all.hpp:29, any.hpp:29) applied to the elements of an expression,
// plus the scalar step that turns the fold into mean, norm2, var or stdev
// (nt2/core/functions/expr/mean.hpp, norm2.hpp, var.hpp, stdev.hpp).  An
// operation supplies its accumulator (state), the neutral state, add,
// merge (the left operand holds the lower indices), warp shuffles, uncached
// loads of partials, and finish(state, n) -> output for a fold of n elements.
enum fin_kind { FIN_NONE = 0, FIN_SQRT = 1, FIN_MEAN = 2 };

template <bool COMP, int FIN = FIN_NONE> struct op_sum {
  template <class T> using state = acc<T>;
  template <class T> using out_t = T;
  template <class T> __device__ __forceinline__ static state<T> init() { return acc<T>{T(0), T(0)}; }
  template <class T> __device__ __forceinline__ static void add(state<T>& a, T x) { fold::add<COMP>(a, x); }
  template <class T> __device__ __forceinline__ static state<T> merge(state<T> a, state<T> b) { return fold::merge<COMP>(a, b); }
  template <class T> __device__ __forceinline__ static state<T> shfl(state<T> a, int off)
  {
    return acc<T>{__shfl_xor_sync(0xffffffffu, a.s, off), __shfl_xor_sync(0xffffffffu, a.c, off)};
  }
  template <class T> __device__ __forceinline__ static state<T> ldcg(const state<T>* p)
  {
    return acc<T>{__ldcg(&p->s), __ldcg(&p->c)};
  }
  template <class T> __device__ __forceinline__ static state<T> shfl_from(state<T> a, int src)
  {
    return acc<T>{__shfl_sync(0xffffffffu, a.s, src), __shfl_sync(0xffffffffu, a.c, src)};
  }
  template <class T> __device__ __forceinline__ static T finish(state<T> a, size_t n)
  {
    const T r = result<COMP>(a);
    if constexpr (FIN == FIN_SQRT) return math::sqrt_(r);
    if constexpr (FIN == FIN_MEAN) return math::mul(math::div(T(1), (T)n), r);   // rec(n) * sum
    return r;
  }
};

template <class T> struct val { T v; };

// max / min / prod: one value; max and min ignore NaNs (NT2's result with NaNs
// depends on its evaluation order), their neutral elements are NT2's Maxinit
// (-largest finite) and Valmax (+largest finite).  KIND 3 and 4 are max and min
// with the neutral elements of cummax and cummin, Minf and Inf
// (boost/simd/swar/functions/cummax.hpp, cummin.hpp).
template <int KIND> struct op_val {   // 0 max, 1 min, 2 prod, 3 cummax, 4 cummin
  template <class T> using state = val<T>;
  template <class T> using out_t = T;
  template <class T> __device__ __forceinline__ static state<T> init()
  {
    // largest finite value: NT2's Valmax, and -Valmax is its Maxinit (constant/constants/maxinit.hpp)
    const T big = sizeof(T) == 4 ? (T)3.40282346638528859812e+38 : (T)1.79769313486231570815e+308;
    const T inf = sizeof(T) == 4 ? (T)__int_as_float(0x7f800000) : (T)__longlong_as_double(0x7ff0000000000000ll);
    if constexpr (KIND == 2) return val<T>{T(1)};
    else if constexpr (KIND == 3) return val<T>{-inf};
    else if constexpr (KIND == 4) return val<T>{inf};
    else return val<T>{KIND == 0 ? -big : big};
  }
  // a is the accumulator (never NaN), b the next element: NT2's max(a,b) = a > b ? a : b
  // (boost/simd/arithmetic/functions/scalar/max.hpp), except that a NaN b is skipped
  template <class T> __device__ __forceinline__ static T op(T a, T b)
  {
    if constexpr (KIND == 0 || KIND == 3) return (a > b || b != b) ? a : b;
    else if constexpr (KIND == 1 || KIND == 4) return (a < b || b != b) ? a : b;
    else return math::mul(a, b);
  }
  template <class T> __device__ __forceinline__ static void add(state<T>& a, T x) { a.v = op(a.v, x); }
  template <class T> __device__ __forceinline__ static state<T> merge(state<T> a, state<T> b) { return val<T>{op(a.v, b.v)}; }
  template <class T> __device__ __forceinline__ static state<T> shfl(state<T> a, int off)
  {
    return val<T>{__shfl_xor_sync(0xffffffffu, a.v, off)};
  }
  template <class T> __device__ __forceinline__ static state<T> ldcg(const state<T>* p) { return val<T>{__ldcg(&p->v)}; }
  template <class T> __device__ __forceinline__ static state<T> shfl_from(state<T> a, int src)
  {
    return val<T>{__shfl_sync(0xffffffffu, a.v, src)};
  }
  template <class T> __device__ __forceinline__ static T finish(state<T> a, size_t) { return a.v; }
};

// all / any: logical_and / logical_or of (x != 0) with neutral True / False;
// none = !any (boost/simd/reduction/functions/scalar/none.hpp: is_eqz of the
// element).  The output is a logical table stored as uint8_t 0/1.
template <bool ANY, bool NOT = false> struct op_logic {
  using flag = val<unsigned>;
  template <class T> using state = flag;
  template <class T> using out_t = uint8_t;
  template <class T> __device__ __forceinline__ static flag init() { return flag{ANY ? 0u : 1u}; }
  template <class T> __device__ __forceinline__ static void add(flag& a, T x)
  {
    const unsigned b = (x != T(0)) ? 1u : 0u;
    a.v = ANY ? (a.v | b) : (a.v & b);
  }
  __device__ __forceinline__ static flag merge(flag a, flag b) { return flag{ANY ? (a.v | b.v) : (a.v & b.v)}; }
  __device__ __forceinline__ static flag shfl(flag a, int off) { return flag{__shfl_xor_sync(0xffffffffu, a.v, off)}; }
  __device__ __forceinline__ static flag ldcg(const flag* p) { return flag{__ldcg(&p->v)}; }
  __device__ __forceinline__ static uint8_t finish(flag a, size_t) { return (uint8_t)(NOT ? (a.v ^ 1u) : a.v); }
};

// var / stdev in one pass: Welford's update per element and Chan's merge of
// partial (count, mean, M2).  NT2 computes var(A) = f * asum2(center(A)) with
// f = rec(n - 1) (rec(n) with w = 1, 1 when n <= 1) in two passes
// (nt2/core/functions/expr/var.hpp); the result here is the same quantity
// within the error bound stated in the tests.
template <class T> struct moments { T n, mean, m2; };

template <bool W1, bool STDEV> struct op_moments {
  template <class U> using state = moments<U>;
  template <class U> using out_t = U;
  template <class U> __device__ __forceinline__ static state<U> init() { return moments<U>{U(0), U(0), U(0)}; }
  template <class U> __device__ __forceinline__ static void add(state<U>& a, U x)
  {
    a.n = a.n + U(1);
    const U d = x - a.mean;
    if constexpr (sizeof(U) == 4) a.mean = __fmaf_rn(d, __frcp_rn(a.n), a.mean);
    else a.mean = a.mean + d / a.n;
    a.m2 = a.m2 + d * (x - a.mean);
  }
  template <class U> __device__ __forceinline__ static state<U> merge(state<U> a, state<U> b)
  {
    if (b.n == U(0)) return a;
    if (a.n == U(0)) return b;
    const U n = a.n + b.n;
    const U d = b.mean - a.mean;
    const U wb = b.n / n;
    return moments<U>{n, a.mean + d * wb, a.m2 + b.m2 + d * d * a.n * wb};
  }
  // N values at once (N a power of two): the block's own mean and sum of
  // squared deviations in two passes over registers, then one merge, so the
  // division of Welford's update is paid once per block instead of per value.
  template <class U, int N> __device__ __forceinline__ static void add_block(state<U>& a, const U (&x)[N])
  {
    static_assert((N & (N - 1)) == 0, "add_block: N a power of two");
    U s = x[0];
#pragma unroll
    for (int i = 1; i < N; ++i) s = s + x[i];
    const U mb = s * (U(1) / U(N));               // exact scaling
    U m2 = U(0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const U d = x[i] - mb;
      m2 = m2 + d * d;
    }
    a = merge(a, moments<U>{U(N), mb, m2});
  }
  template <class U> __device__ __forceinline__ static state<U> shfl(state<U> a, int off)
  {
    return moments<U>{__shfl_xor_sync(0xffffffffu, a.n, off), __shfl_xor_sync(0xffffffffu, a.mean, off),
                      __shfl_xor_sync(0xffffffffu, a.m2, off)};
  }
  template <class U> __device__ __forceinline__ static state<U> ldcg(const state<U>* p)
  {
    return moments<U>{__ldcg(&p->n), __ldcg(&p->mean), __ldcg(&p->m2)};
  }
  template <class U> __device__ __forceinline__ static U finish(state<U> a, size_t n)
  {
    const U n1 = (U)n - (W1 ? U(0) : U(1));
    const U f = (n <= 1) ? U(1) : math::div(U(1), n1);
    const U v = math::mul(f, a.m2);
    return STDEV ? math::sqrt_(v) : v;
  }
};

template <class Op, class T> using state_of = typename Op::template state<T>;

// Operations that take a block of values at once (add_block).
template <class Op> struct has_block_add { static constexpr bool value = false; };
template <bool W1, bool SD> struct has_block_add<op_moments<W1, SD>> { static constexpr bool value = true; };
template <class Op, class T> using out_of = typename Op::template out_t<T>;

// Butterfly over the warp; every lane ends with the same value.
template <class Op, class T> __device__ __forceinline__ state_of<Op, T> warp_merge(state_of<Op, T> a)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    state_of<Op, T> o = Op::shfl(a, off);
    // combine in lane order so every lane computes the same value
    a = ((threadIdx.x & 31) & off) ? Op::merge(o, a) : Op::merge(a, o);
  }
  return a;
}

// Folds of zero elements: every output is finish(neutral).
template <class Op, class T>
__global__ void __launch_bounds__(256) k_fold_empty(out_of<Op, T>* __restrict__ out, size_t count)
{
  nt2cuda::mem::pdl_begin();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    out[i] = Op::finish(Op::template init<T>(), 0);
}

// ------------------------------------------------------------ inner fold
// Work unit: one warp reduces the segment [r0, r1) of column j, where the
// column is split into `splits` segments of `seg` elements (seg a multiple
// of 32*V).  With splits > 1 the warp writes its partial to scratch and the
// last warp of the column combines the column's partials in segment order.
struct inner_shape {
  size_t rows, cols, seg, splits;
};

template <class Op, int V, int U, class T, class E>
__global__ void __launch_bounds__(256) k_inner(E e, inner_shape sh, out_of<Op, T>* __restrict__ out,
                                               state_of<Op, T>* __restrict__ partials, unsigned* __restrict__ counters)
{
  const int lane = threadIdx.x & 31;
  const size_t warps_total = (size_t)gridDim.x * (blockDim.x >> 5);
  const size_t units = sh.cols * sh.splits;
  {
    // while the previous grid drains, have the L2 fetch the lines of this
    // warp's first U loads (one prefetch per 128-byte line)
    const size_t w = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    constexpr int LANES_PER_LINE = (V * (int)sizeof(T)) >= 128 ? 1 : 128 / (V * (int)sizeof(T));
    if (w < units && V > 1 && lane % LANES_PER_LINE == 0) {
      const size_t j = w / sh.splits, r0 = (w % sh.splits) * sh.seg;
      const size_t r1 = (r0 + sh.seg < sh.rows) ? r0 + sh.seg : sh.rows;
      const size_t g1 = r1 / V;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const size_t g = r0 / V + lane + (size_t)u * 32;
        if (g < g1) prefetch_terms(e, j * sh.rows + g * V);
      }
    }
  }
  nt2cuda::mem::pdl_begin();
  for (size_t w = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < units; w += warps_total) {
    const size_t j = w / sh.splits, sp = w % sh.splits;
    const size_t r0 = sp * sh.seg;
    const size_t r1 = (r0 + sh.seg < sh.rows) ? r0 + sh.seg : sh.rows;
    const size_t base = j * sh.rows;
    state_of<Op, T> a[V];
#pragma unroll
    for (int l = 0; l < V; ++l) a[l] = Op::template init<T>();
    // full V-groups
    const size_t g0 = r0 / V, g1 = r1 / V;   // r0 is a multiple of V
    size_t g = g0 + lane;
    for (; g + (size_t)(U - 1) * 32 < g1; g += (size_t)U * 32) {
      regs<E, V> rr[U];
#pragma unroll
      for (int u = 0; u < U; ++u) rr[u].template load<true>(e, base + (g + (size_t)u * 32) * V);
      if constexpr (has_block_add<Op>::value && ((U * V) & (U * V - 1)) == 0) {
        T blk[U * V];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int l = 0; l < V; ++l) blk[u * V + l] = (T)rr[u].template get<false>(e, l);
        Op::add_block(a[0], blk);
      } else {
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int l = 0; l < V; ++l) Op::add(a[l], (T)rr[u].template get<false>(e, l));
      }
    }
    for (; g < g1; g += 32) {
      regs<E, V> rr;
      rr.template load<true>(e, base + g * V);
#pragma unroll
      for (int l = 0; l < V; ++l) Op::add(a[l], (T)rr.template get<false>(e, l));
    }
    // ragged end of the segment (only when rows % V != 0 or V == 1)
    for (size_t r = g1 * V + lane; r < r1; r += 32) {
      regs<E, 1> rr;
      rr.template load<false>(e, base + r);
      Op::add(a[0], (T)rr.template get<false>(e, 0));
    }
    state_of<Op, T> t = a[0];
#pragma unroll
    for (int l = 1; l < V; ++l) t = Op::merge(t, a[l]);
    t = warp_merge<Op, T>(t);
    if (sh.splits == 1) {
      if (lane == 0) out[j] = Op::finish(t, sh.rows);
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
    state_of<Op, T> c = Op::template init<T>();
    for (size_t q = lane; q < sh.splits; q += 32) c = Op::merge(c, Op::ldcg(partials + j * sh.splits + q));
    c = warp_merge<Op, T>(c);
    if (lane == 0) out[j] = Op::finish(c, sh.rows);
  }
}

// Short columns (rows < 32): one thread folds one whole column.
template <class Op, class T, class E>
__global__ void __launch_bounds__(256) k_inner_short(E e, size_t rows, size_t cols, out_of<Op, T>* __restrict__ out)
{
  nt2cuda::mem::pdl_begin();
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < cols; j += (size_t)gridDim.x * blockDim.x) {
    state_of<Op, T> a = Op::template init<T>();
    for (size_t r = 0; r < rows; ++r) {
      regs<E, 1> rr;
      rr.template load<false>(e, j * rows + r);
      Op::add(a, (T)rr.template get<false>(e, 0));
    }
    out[j] = Op::finish(a, rows);
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

template <class Op, int V, int U, class T, class E>
__global__ void __launch_bounds__(256) k_outer(E e, outer_shape sh, out_of<Op, T>* __restrict__ out,
                                               state_of<Op, T>* __restrict__ partials, unsigned* __restrict__ counters)
{
  using S = state_of<Op, T>;
  constexpr int STRIP = 32 * V;
  __shared__ S red[8][STRIP];
  __shared__ unsigned is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t units = sh.strips * sh.splits;
  {
    // while the previous grid drains, have the L2 fetch the lines of this
    // warp's first U loads of its first unit (one prefetch per 128-byte line)
    constexpr int LANES_PER_LINE = (V * (int)sizeof(T)) >= 128 ? 1 : 128 / (V * (int)sizeof(T));
    const size_t b = blockIdx.x;
    if (b < units && V > 1 && lane % LANES_PER_LINE == 0) {
      const size_t strip = b / sh.splits, m0 = (b % sh.splits) * sh.cchunk;
      const size_t row0 = strip * STRIP + (size_t)lane * V;
      const size_t m1 = (m0 + sh.cchunk < sh.cols) ? m0 + sh.cchunk : sh.cols;
      if (row0 + V <= sh.rows) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const size_t m = m0 + warp + (size_t)u * 8;
          if (m < m1) prefetch_terms(e, m * sh.rows + row0);
        }
      }
    }
  }
  nt2cuda::mem::pdl_begin();
  for (size_t b = blockIdx.x; b < units; b += gridDim.x) {
    const size_t strip = b / sh.splits, sp = b % sh.splits;
    const size_t row0 = strip * STRIP + (size_t)lane * V;   // first row of this lane
    const size_t m0 = sp * sh.cchunk;
    const size_t m1 = (m0 + sh.cchunk < sh.cols) ? m0 + sh.cchunk : sh.cols;
    const bool full = row0 + V <= sh.rows;
    S a[V];
#pragma unroll
    for (int l = 0; l < V; ++l) a[l] = Op::template init<T>();
    if (full) {
      size_t m = m0 + warp;
      for (; m + (size_t)(U - 1) * 8 < m1; m += (size_t)U * 8) {
        regs<E, V> rr[U];
#pragma unroll
        for (int u = 0; u < U; ++u) rr[u].template load<true>(e, (m + (size_t)u * 8) * sh.rows + row0);
        if constexpr (has_block_add<Op>::value && (U & (U - 1)) == 0) {
          // lane slot l is one row: its U values of this trip form a block
#pragma unroll
          for (int l = 0; l < V; ++l) {
            T blk[U];
#pragma unroll
            for (int u = 0; u < U; ++u) blk[u] = (T)rr[u].template get<false>(e, l);
            Op::add_block(a[l], blk);
          }
        } else {
#pragma unroll
          for (int u = 0; u < U; ++u)
#pragma unroll
            for (int l = 0; l < V; ++l) Op::add(a[l], (T)rr[u].template get<false>(e, l));
        }
      }
      for (; m < m1; m += 8) {
        regs<E, V> rr;
        rr.template load<true>(e, m * sh.rows + row0);
#pragma unroll
        for (int l = 0; l < V; ++l) Op::add(a[l], (T)rr.template get<false>(e, l));
      }
    } else if (row0 < sh.rows) {
      for (size_t m = m0 + warp; m < m1; m += 8)
#pragma unroll
        for (int l = 0; l < V; ++l)
          if (row0 + l < sh.rows) {
            regs<E, 1> rr;
            rr.template load<false>(e, m * sh.rows + row0 + l);
            Op::add(a[l], (T)rr.template get<false>(e, 0));
          }
    }
#pragma unroll
    for (int l = 0; l < V; ++l) red[warp][lane * V + l] = a[l];
    __syncthreads();
    // thread t < STRIP merges row t of the strip over the 8 warps in order
    S rsum = Op::template init<T>();
    const size_t row = strip * STRIP + threadIdx.x;
    if (threadIdx.x < STRIP) {
      rsum = red[0][threadIdx.x];
#pragma unroll
      for (int w = 1; w < 8; ++w) rsum = Op::merge(rsum, red[w][threadIdx.x]);
    }
    if (sh.splits == 1) {
      if (threadIdx.x < STRIP && row < sh.rows) out[row] = Op::finish(rsum, sh.cols);
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
        S c = Op::template init<T>();
        size_t q = 0;
        for (; q + 8 <= sh.splits; q += 8) {
          S v[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) v[k] = Op::ldcg(partials + (strip * sh.splits + q + k) * STRIP + threadIdx.x);
#pragma unroll
          for (int k = 0; k < 8; ++k) c = Op::merge(c, v[k]);
        }
        for (; q < sh.splits; ++q) c = Op::merge(c, Op::ldcg(partials + (strip * sh.splits + q) * STRIP + threadIdx.x));
        out[row] = Op::finish(c, sh.cols);
      }
    }
    __syncthreads();
  }
}

}  // namespace fold
}  // namespace nt2cuda
