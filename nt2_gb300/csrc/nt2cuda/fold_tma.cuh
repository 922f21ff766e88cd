// nt2cuda/fold_tma.cuh -- inner_fold and outer_fold with TMA-staged tiles.
//
// Same results contract as fold.cuh (any of its reduction operations,
// partials merged in index order, decomposition fixed by the table's shape),
// but the input tiles reach shared memory through the Tensor Memory
// Accelerator, so each block keeps several 16 KB tiles in flight without
// holding them in registers:
//   inner_fold (sum(A,1), globalsum, globalsum(X*Y)): a unit is one segment of
//     one column; its tiles are contiguous, one 1-D cp.async.bulk per term.
//   outer_fold (sum(A,2)): a unit is a strip of 256 rows by a chunk of columns;
//     each tile is a 256-row x 16-column box loaded through a 2-D tensor map,
//     which also zero-fills the ragged edges of the table.
// NT2's counterparts: modules/arch/shared_memory/include/nt2/sdk/shared_memory/worker/inner_fold.hpp:53-108
// and .../worker/outer_fold.hpp:31-155.
//
// A block whose barrier wait runs out (tma::mbar_wait) waits (bounded) for
// the copies it still has in flight, counts itself in g_fold_wait_timeouts
// (read by nt2cuda_wait_timeouts) and gives up the units it still owns: a unit
// of a column or strip that is folded in one piece gets NaN at once; a split
// one still arrives on its column's counter with the poison bit set, so the
// counter returns to zero as in a complete fold and the last arriver writes
// NaN instead of merging partials that were never written.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <mutex>
#include "fold.cuh"
#include "launch.cuh"
#include "scratch.cuh"
#include "tma.cuh"
#include "wait_status.cuh"

namespace nt2cuda {
namespace fold {

constexpr int kTmaTileBytes = 16384;

// Barrier waits of these kernels that ran out since this translation unit was
// loaded; every unit including this header registers a reader (fold_status.hpp).
static __device__ unsigned long long g_fold_wait_timeouts = 0;
static cudaError_t read_fold_wait_timeouts(unsigned long long* count)
{
  return cudaMemcpyFromSymbol(count, g_fold_wait_timeouts, sizeof(unsigned long long));
}
static const timeout_reader_registration fold_wait_timeouts_reader(read_fold_wait_timeouts);

// Arrival counters: the low 31 bits count the units merged so far, the top bit
// records that a unit of the column gave up.
constexpr unsigned kPoison = 0x80000000u;
__device__ __forceinline__ unsigned arrive(unsigned* counter, bool poisoned)
{
  if (poisoned) atomicOr(counter, kPoison);
  return atomicAdd(counter, 1u);
}

// value written for a unit whose copies did not arrive: NaN, or 0xFF for a logical output
template <class T> __device__ __forceinline__ T quiet_nan()
{
  if constexpr (sizeof(T) == 1) return (T)0xFF;
  else if constexpr (sizeof(T) == 4) return __int_as_float(0x7fc00000);
  else return __longlong_as_double(0x7ff8000000000000ll);
}

// Merge n partials p[0], p[stride], ... in index order, with 8 loads in
// flight at a time (the merge is at the tail of the kernel, where serial L2
// round trips would show).
template <class Op, class T>
__device__ __forceinline__ state_of<Op, T> merge_partials(const state_of<Op, T>* p, size_t n, size_t stride)
{
  state_of<Op, T> m = Op::template init<T>();
  size_t q = 0;
  for (; q + 8 <= n; q += 8) {
    state_of<Op, T> v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = Op::ldcg(p + (q + k) * stride);
#pragma unroll
    for (int k = 0; k < 8; ++k) m = Op::merge(m, v[k]);
  }
  for (; q < n; ++q) m = Op::merge(m, Op::ldcg(p + q * stride));
  return m;
}

// Merge v[threadIdx.x] over the block in a fixed order; thread 0 gets the result.
template <class Op, class T>
__device__ __forceinline__ state_of<Op, T> block_merge(state_of<Op, T> v, state_of<Op, T>* red)
{
  v = warp_merge<Op, T>(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  state_of<Op, T> r = red[0];
  if (threadIdx.x == 0)
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = Op::merge(r, red[w]);
  __syncthreads();
  return r;
}

// ------------------------------------------------------------ inner fold
// fail_unit: the unit whose first tile the producer arms but never copies, so
// that its barrier wait runs out (~0 in every fold; set only by the timeout
// self-test); wait_rounds bounds every barrier wait.
struct inner_tma_shape {
  size_t rows, cols, seg, splits, units;
  size_t fail_unit;
  uint32_t wait_rounds;
};

// A block that gave up: count it, then let every unit it still owns arrive
// poisoned (a column folded in one piece gets NaN at once; a split column's
// last arriver writes NaN and clears the counter).  Every thread of the block
// calls this with the same first unit.
template <class O>
__device__ void inner_give_up(const inner_tma_shape& sh, size_t cu, O* out, unsigned* counters)
{
  if (threadIdx.x != 0) return;
  atomicAdd(&g_fold_wait_timeouts, 1ull);
  for (size_t u = cu; u < sh.units; u += gridDim.x) {
    const size_t j = u / sh.splits;
    if (sh.splits == 1) {
      out[j] = quiet_nan<O>();
    } else {
      const unsigned prev = arrive(&counters[j], true);
      if ((prev & ~kPoison) == (unsigned)sh.splits - 1u) {
        counters[j] = 0u;
        out[j] = quiet_nan<O>();
      }
    }
  }
}

template <class T> __host__ __device__ constexpr int inner_tile() { return kTmaTileBytes / (int)sizeof(T); }

template <class T>
__device__ __forceinline__ size_t inner_unit_tiles(const inner_tma_shape& sh, size_t u)
{
  const size_t r0 = (u % sh.splits) * sh.seg;
  const size_t r1 = (r0 + sh.seg < sh.rows) ? r0 + sh.seg : sh.rows;
  return (r1 - r0 + inner_tile<T>() - 1) / inner_tile<T>();
}

// NT = 1 folds x; NT = 2 folds x*y (float product rounded, as NT2's X*Y).
template <class Op, class T, int NT, int STAGES>
__global__ void __launch_bounds__(256) k_inner_tma(const T* __restrict__ x, const T* __restrict__ y,
                                                   inner_tma_shape sh, out_of<Op, T>* __restrict__ out,
                                                   state_of<Op, T>* __restrict__ partials,
                                                   unsigned* __restrict__ counters)
{
  using S = state_of<Op, T>;
  constexpr int TILE = inner_tile<T>();
  constexpr int V = 16 / (int)sizeof(T);
  if (blockIdx.x < sh.units) {
    // while the previous grid drains, have the L2 fetch the first STAGES tiles
    // of this block's first unit (one prefetch per 128-byte line)
    const size_t u = blockIdx.x, j = u / sh.splits, r0 = (u % sh.splits) * sh.seg;
    const size_t rend = (r0 + sh.seg < sh.rows) ? r0 + sh.seg : sh.rows;
    const size_t span = (rend - r0 < (size_t)STAGES * TILE) ? rend - r0 : (size_t)STAGES * TILE;
    const size_t lines = (span * sizeof(T) + 127) / 128;
    for (size_t q = threadIdx.x; q < lines; q += blockDim.x) {
      nt2cuda::mem::prefetch_l2(reinterpret_cast<const char*>(x + j * sh.rows + r0) + q * 128);
      if constexpr (NT == 2) nt2cuda::mem::prefetch_l2(reinterpret_cast<const char*>(y + j * sh.rows + r0) + q * 128);
    }
  }
  nt2cuda::mem::pdl_begin();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* buf = reinterpret_cast<T*>(smem_raw);          // [STAGES][NT][TILE]
  __shared__ __align__(8) uint64_t bar[STAGES];
  __shared__ S red[8];
  __shared__ unsigned s_last;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) tma::mbar_init(&bar[s], 1);
    tma::fence_barrier_init();
  }
  __syncthreads();

  // producer state (thread 0): next tile to issue
  size_t pu = blockIdx.x, pt = 0;
  uint32_t issued = 0;
  auto produce = [&](int s) {
    const size_t j = pu / sh.splits, r0 = (pu % sh.splits) * sh.seg + pt * (size_t)TILE;
    const size_t rend = ((pu % sh.splits) * sh.seg + sh.seg < sh.rows) ? (pu % sh.splits) * sh.seg + sh.seg : sh.rows;
    const uint32_t cnt = (uint32_t)((rend - r0) < (size_t)TILE ? (rend - r0) : (size_t)TILE);
    const uint32_t bytes = cnt * (uint32_t)sizeof(T);
    tma::mbar_arrive_expect_tx(&bar[s], bytes * NT);
    if (!(pu == sh.fail_unit && pt == 0)) {
      tma::bulk_g2s(buf + (size_t)(s * NT) * TILE, x + j * sh.rows + r0, bytes, &bar[s]);
      if constexpr (NT == 2) tma::bulk_g2s(buf + (size_t)(s * NT + 1) * TILE, y + j * sh.rows + r0, bytes, &bar[s]);
    }
    ++issued;
    if (++pt == inner_unit_tiles<T>(sh, pu)) { pt = 0; pu += gridDim.x; }
  };
  if (threadIdx.x == 0)
    for (int s = 0; s < STAGES && pu < sh.units; ++s) produce(s);

  size_t cu = blockIdx.x, ct = 0;
  uint32_t iter = 0;
  S a[V];
#pragma unroll
  for (int l = 0; l < V; ++l) a[l] = Op::template init<T>();
  while (cu < sh.units) {
    const int s = (int)(iter % STAGES);
    const bool ok = tma::mbar_wait(&bar[s], (iter / STAGES) & 1u, sh.wait_rounds);
    if (__syncthreads_or(!ok)) {
      // copies still in flight land in this block's shared memory: wait for
      // them (bounded) before leaving, the one that ran out included
      if (threadIdx.x == 0)
        for (uint32_t k = iter; k < issued; ++k) tma::mbar_wait(&bar[k % STAGES], (k / STAGES) & 1u, sh.wait_rounds);
      inner_give_up(sh, cu, out, counters);
      __syncthreads();
      return;
    }
    const size_t j = cu / sh.splits;
    const size_t seg0 = (cu % sh.splits) * sh.seg;
    const size_t rend = (seg0 + sh.seg < sh.rows) ? seg0 + sh.seg : sh.rows;
    const size_t r0 = seg0 + ct * (size_t)TILE;
    const int cnt = (int)((rend - r0) < (size_t)TILE ? (rend - r0) : (size_t)TILE);
    const T* tx = buf + (size_t)(s * NT) * TILE;
    const T* ty = buf + (size_t)(s * NT + (NT == 2 ? 1 : 0)) * TILE;
    for (int e = threadIdx.x * V; e < cnt; e += 256 * V) {
      T xv[V];
      *reinterpret_cast<uint4*>(xv) = *reinterpret_cast<const uint4*>(tx + e);
      if constexpr (NT == 2) {
        T yv[V];
        *reinterpret_cast<uint4*>(yv) = *reinterpret_cast<const uint4*>(ty + e);
#pragma unroll
        for (int l = 0; l < V; ++l) Op::add(a[l], math::mul(xv[l], yv[l]));
      } else if constexpr (has_block_add<Op>::value) {
        Op::add_block(a[0], xv);                       // var/stdev: one merge per V values
      } else {
#pragma unroll
        for (int l = 0; l < V; ++l) Op::add(a[l], xv[l]);
      }
    }
    __syncthreads();                                   // every thread is done with stage s
    if (threadIdx.x == 0 && pu < sh.units) {
      tma::fence_proxy_async();
      produce(s);
    }
    if (++ct == inner_unit_tiles<T>(sh, cu)) {         // unit complete: merge and emit
      S t = a[0];
#pragma unroll
      for (int l = 1; l < V; ++l) t = Op::merge(t, a[l]);
      t = block_merge<Op, T>(t, red);
      if (sh.splits == 1) {
        if (threadIdx.x == 0) out[j] = Op::finish(t, sh.rows);
      } else {
        if (threadIdx.x == 0) {
          partials[cu] = t;
          __threadfence();
          const unsigned prev = arrive(&counters[j], false);
          s_last = ((prev & ~kPoison) == (unsigned)sh.splits - 1u) ? 1u + (prev >> 31) : 0u;
          if (s_last) counters[j] = 0u;
        }
        __syncthreads();
        if (s_last == 2u) {                            // a unit of this column gave up
          if (threadIdx.x == 0) out[j] = quiet_nan<out_of<Op, T>>();
        } else if (s_last) {
          __threadfence();
          S m = Op::template init<T>();
          for (size_t q = threadIdx.x; q < sh.splits; q += blockDim.x)
            m = Op::merge(m, Op::ldcg(partials + j * sh.splits + q));
          m = block_merge<Op, T>(m, red);
          if (threadIdx.x == 0) out[j] = Op::finish(m, sh.rows);
        }
      }
#pragma unroll
      for (int l = 0; l < V; ++l) a[l] = Op::template init<T>();
      ct = 0;
      cu += gridDim.x;
    }
    ++iter;
  }
}

// ------------------------------------------------------------ outer fold
struct outer_tma_shape {
  size_t rows, cols, cchunk, splits, strips, units;
  uint32_t wait_rounds;
};

constexpr int kOuterRows = 256;   // box rows (and threads per block)
template <class T> __host__ __device__ constexpr int outer_cols() { return kTmaTileBytes / (kOuterRows * (int)sizeof(T)); }

template <class Op, class T, int STAGES>
__global__ void __launch_bounds__(256) k_outer_tma(const __grid_constant__ CUtensorMap map, outer_tma_shape sh,
                                                   out_of<Op, T>* __restrict__ out,
                                                   state_of<Op, T>* __restrict__ partials,
                                                   unsigned* __restrict__ counters)
{
  nt2cuda::mem::pdl_begin();
  using S = state_of<Op, T>;
  constexpr int BR = kOuterRows, BC = outer_cols<T>();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* buf = reinterpret_cast<T*>(smem_raw);          // [STAGES][BC][BR]
  __shared__ __align__(8) uint64_t bar[STAGES];
  __shared__ unsigned s_last;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) tma::mbar_init(&bar[s], 1);
    tma::fence_barrier_init();
  }
  __syncthreads();

  auto unit_tiles = [&](size_t u) {
    const size_t c0 = (u % sh.splits) * sh.cchunk;
    const size_t c1 = (c0 + sh.cchunk < sh.cols) ? c0 + sh.cchunk : sh.cols;
    return (c1 - c0 + BC - 1) / BC;
  };
  size_t pu = blockIdx.x, pt = 0;
  uint32_t issued = 0;
  auto produce = [&](int s) {
    const int xr = (int)((pu / sh.splits) * BR);
    const int yc = (int)((pu % sh.splits) * sh.cchunk + pt * BC);
    tma::mbar_arrive_expect_tx(&bar[s], (uint32_t)(BR * BC * sizeof(T)));
    tma::tensor_g2s_2d(buf + (size_t)s * BC * BR, &map, xr, yc, &bar[s]);
    ++issued;
    if (++pt == unit_tiles(pu)) { pt = 0; pu += gridDim.x; }
  };
  if (threadIdx.x == 0)
    for (int s = 0; s < STAGES && pu < sh.units; ++s) produce(s);

  size_t cu = blockIdx.x, ct = 0;
  uint32_t iter = 0;
  S a0 = Op::template init<T>(), a1 = Op::template init<T>();
  while (cu < sh.units) {
    const int s = (int)(iter % STAGES);
    const bool ok = tma::mbar_wait(&bar[s], (iter / STAGES) & 1u, sh.wait_rounds);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        for (uint32_t k = iter; k < issued; ++k) tma::mbar_wait(&bar[k % STAGES], (k / STAGES) & 1u, sh.wait_rounds);
        atomicAdd(&g_fold_wait_timeouts, 1ull);
      }
      // every unit this block still owns arrives poisoned (see inner_give_up)
      for (size_t u = cu; u < sh.units; u += gridDim.x) {
        const size_t strip = u / sh.splits;
        if (sh.splits > 1) {
          if (threadIdx.x == 0) {
            const unsigned prev = arrive(&counters[strip], true);
            s_last = ((prev & ~kPoison) == (unsigned)sh.splits - 1u) ? 1u : 0u;
            if (s_last) counters[strip] = 0u;
          }
          __syncthreads();
        }
        const bool last = sh.splits == 1 || s_last;
        const size_t row = strip * BR + threadIdx.x;
        if (last && row < sh.rows) out[row] = quiet_nan<out_of<Op, T>>();
        __syncthreads();
      }
      return;
    }
    const T* tile = buf + (size_t)s * BC * BR;
    // columns past the table are zero-filled by the copy and skipped (a zero is
    // not neutral for every operation); chunks are whole tiles wide
    const size_t cbase = (cu % sh.splits) * sh.cchunk + ct * BC;
    if (cbase + BC <= sh.cols) {
#pragma unroll
      for (int c = 0; c < BC; c += 2) {
        Op::add(a0, tile[c * BR + threadIdx.x]);
        Op::add(a1, tile[(c + 1) * BR + threadIdx.x]);
      }
    } else {
      for (int c = 0; c < BC; ++c)
        if (cbase + c < sh.cols) Op::add((c & 1) ? a1 : a0, tile[c * BR + threadIdx.x]);
    }
    __syncthreads();
    if (threadIdx.x == 0 && pu < sh.units) {
      tma::fence_proxy_async();
      produce(s);
    }
    if (++ct == unit_tiles(cu)) {
      const size_t strip = cu / sh.splits;
      const size_t row = strip * BR + threadIdx.x;
      const S t = Op::merge(a0, a1);
      if (sh.splits == 1) {
        if (row < sh.rows) out[row] = Op::finish(t, sh.cols);
      } else {
        partials[cu * BR + threadIdx.x] = t;
        __syncthreads();                    // the block's partials, then one device-scope fence
        if (threadIdx.x == 0) {
          __threadfence();
          const unsigned prev = arrive(&counters[strip], false);
          s_last = ((prev & ~kPoison) == (unsigned)sh.splits - 1u) ? 1u + (prev >> 31) : 0u;
          if (s_last) counters[strip] = 0u;
        }
        __syncthreads();
        if (s_last == 2u) {                  // a unit of this strip gave up
          if (row < sh.rows) out[row] = quiet_nan<out_of<Op, T>>();
        } else if (s_last) {
          __threadfence();
          S m = merge_partials<Op, T>(partials + strip * sh.splits * BR + threadIdx.x, sh.splits, BR);
          if (row < sh.rows) out[row] = Op::finish(m, sh.cols);
        }
      }
      a0 = Op::template init<T>();
      a1 = Op::template init<T>();
      ct = 0;
      cu += gridDim.x;
    }
    ++iter;
  }
}

// ------------------------------------------------------------- launchers
using tma::tensor_map_encoder;

template <class K> inline cudaError_t set_smem(K kernel, int bytes)
{
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// x (and y when not null) are 16-byte aligned and rows % (16/sizeof(T)) == 0.
// fail_unit and wait_rounds are for the timeout self-test (see inner_tma_shape).
template <class Op, class T>
cudaError_t inner_fold_tma(const T* x, const T* y, size_t rows, size_t cols, out_of<Op, T>* out, cudaStream_t s,
                           size_t fail_unit = ~(size_t)0, uint32_t wait_rounds = tma::kMaxRounds)
{
  using S = state_of<Op, T>;
  constexpr int TILE = inner_tile<T>();
  inner_tma_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.seg = (size_t)TILE * 16;
  sh.splits = (rows + sh.seg - 1) / sh.seg;
  sh.units = cols * sh.splits;
  sh.fail_unit = fail_unit;
  sh.wait_rounds = wait_rounds;
  if (sh.units == 0) return cudaSuccess;
  S* partials = nullptr;
  unsigned* counters = nullptr;
  if (sh.splits > 1) {
    void* p = nullptr;
    cudaError_t e = fold_scratch(s, cols, sh.units, sizeof(S), &counters, &p);
    if (e != cudaSuccess) return e;
    partials = (S*)p;
  }
  size_t grid;
  cudaError_t e;
  if (y) {
    constexpr int ST = 3;
    auto k = k_inner_tma<Op, T, 2, ST>;
    const int smem = ST * 2 * kTmaTileBytes;
    if ((e = set_smem(k, smem)) != cudaSuccess) return e;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 256, smem);
    grid = (size_t)sm_count() * (size_t)(per > 0 ? per : 1);
    if (grid > sh.units) grid = sh.units;
    void* args[] = {(void*)&x, (void*)&y, (void*)&sh, (void*)&out, (void*)&partials, (void*)&counters};
    e = launch_dependent(k, grid, 256, s, args, smem);
    if (e != cudaSuccess) return e;
  } else {
    constexpr int ST = 4;
    auto k = k_inner_tma<Op, T, 1, ST>;
    const int smem = ST * kTmaTileBytes;
    if ((e = set_smem(k, smem)) != cudaSuccess) return e;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 256, smem);
    grid = (size_t)sm_count() * (size_t)(per > 0 ? per : 1);
    if (grid > sh.units) grid = sh.units;
    void* args[] = {(void*)&x, (void*)&y, (void*)&sh, (void*)&out, (void*)&partials, (void*)&counters};
    e = launch_dependent(k, grid, 256, s, args, smem);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// A is 16-byte aligned and rows % (16/sizeof(T)) == 0; rows, cols < 2^31.
template <class Op, class T>
cudaError_t outer_fold_tma(const T* A, size_t rows, size_t cols, out_of<Op, T>* out, cudaStream_t s)
{
  using S = state_of<Op, T>;
  constexpr int BR = kOuterRows, BC = outer_cols<T>();
  if (rows == 0 || cols == 0) return cudaSuccess;
  if (rows >= ((size_t)1 << 31) || cols >= ((size_t)1 << 31)) return cudaErrorNotSupported;
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return cudaErrorNotSupported;
  CUtensorMap map;
  const cuuint64_t gdim[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  const cuuint64_t gstride[1] = {(cuuint64_t)rows * sizeof(T)};
  const cuuint32_t box[2] = {(cuuint32_t)BR, (cuuint32_t)BC};
  const cuuint32_t estride[2] = {1, 1};
  CUresult r = encode(&map, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2,
                      (void*)A, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  outer_tma_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.strips = (rows + BR - 1) / BR;
  // about 2048 units so blocks stay balanced; a chunk is a whole number of tiles
  size_t want = (cols * sh.strips + 2047) / 2048;
  sh.cchunk = ((want + BC - 1) / BC) * BC;
  if (sh.cchunk < (size_t)BC) sh.cchunk = BC;
  sh.splits = (cols + sh.cchunk - 1) / sh.cchunk;
  sh.units = sh.strips * sh.splits;
  sh.wait_rounds = tma::kMaxRounds;
  S* partials = nullptr;
  unsigned* counters = nullptr;
  if (sh.splits > 1) {
    void* p = nullptr;
    cudaError_t e = fold_scratch(s, sh.strips, sh.units * BR, sizeof(S), &counters, &p);
    if (e != cudaSuccess) return e;
    partials = (S*)p;
  }
  constexpr int ST = 4;
  auto k = k_outer_tma<Op, T, ST>;
  const int smem = ST * kTmaTileBytes;
  cudaError_t e = set_smem(k, smem);
  if (e != cudaSuccess) return e;
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 256, smem);
  size_t grid = (size_t)sm_count() * (size_t)(per > 0 ? per : 1);
  if (grid > sh.units) grid = sh.units;
  void* args[] = {(void*)&map, (void*)&sh, (void*)&out, (void*)&partials, (void*)&counters};
  e = launch_dependent(k, grid, 256, s, args, smem);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace fold
}  // namespace nt2cuda
