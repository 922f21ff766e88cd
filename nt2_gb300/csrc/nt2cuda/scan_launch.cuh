// nt2cuda/scan_launch.cuh -- host launchers of the scan kernels (scan.cuh):
// inner_scan (along dim 1) and outer_scan (along dim 2) of a column-major
// table, out-of-place or in place.  The NT2 overloads they replace are
// modules/arch/shared_memory/include/nt2/core/functions/shared_memory/{inner,outer}_scan.hpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "launch.cuh"
#include "scan.cuh"
#include "scratch.cuh"
#include "wait_status.cuh"

namespace nt2cuda {
namespace scan {

inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

template <class Op, class T>
cudaError_t inner_scan(const T* x, T* y, size_t rows, size_t cols, cudaStream_t s)
{
  using S = state_of<Op, T>;
  if (!rows || !cols) return cudaSuccess;
  if (rows <= 64) {
    void* args[] = {(void*)&x, (void*)&y, (void*)&rows, (void*)&cols};
    return launch_persistent(k_scan_inner_short<Op, T>, cols, 256, 2, s, args);
  }
  // columns of one 32 KB tile: a single pass without look-back; longer ones:
  // 64 KB tiles chained by the look-back, aggregate then rescan from L2
  const bool one_pass = rows <= (size_t)tile<T>();
  const size_t TILE = one_pass ? (size_t)tile<T>() : scan_tiles<Op, T>::TILE;
  inner_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.tiles_per_col = (rows + TILE - 1) / TILE;
  sh.tiles = sh.tiles_per_col * cols;
  // scratch: ticket, error word, flags | aggregates | inclusive prefixes
  const size_t head = 256, fbytes = align256(sh.tiles * sizeof(unsigned));
  const size_t sbytes = align256(sh.tiles * carry_bytes<Op, T>());
  void* scratch = nullptr;
  cudaError_t e = nt2cuda::stream_scratch(s, head + fbytes + 2 * sbytes, &scratch, 1);
  if (e != cudaSuccess) return e;
  char* b = (char*)scratch;
  unsigned long long* ticket = (unsigned long long*)b;
  unsigned* err = (unsigned*)(b + 8);
  unsigned* flags = (unsigned*)(b + head);
  void* agg = b + head + fbytes;
  void* incl = b + head + fbytes + sbytes;
  if ((e = cudaMemsetAsync(b, 0, head + fbytes, s)) != cudaSuccess) return e;
  int vec = ((((uintptr_t)x | (uintptr_t)y) & 15u) == 0 && (rows * sizeof(T)) % 16 == 0) ? 1 : 0;
  auto k = one_pass ? k_scan_inner_1p<Op, T> : k_scan_inner<Op, T>;
  size_t grid = (size_t)sm_count() * (size_t)resident_blocks(k, 256);
  if (grid > sh.tiles) grid = sh.tiles;
  void* args[] = {(void*)&x, (void*)&y, (void*)&sh, (void*)&vec, (void*)&ticket, (void*)&flags, (void*)&agg,
                  (void*)&incl, (void*)&err};
  return launch_dependent(k, grid, 256, s, args);
}

static cudaError_t read_scan_wait_timeouts(unsigned long long* count)
{
  return cudaMemcpyFromSymbol(count, g_wait_timeouts, sizeof(unsigned long long));
}
static const timeout_reader_registration scan_wait_timeouts_reader(read_scan_wait_timeouts);

// Bounded waits that ran out since the library was loaded, over every kernel
// that counts them (scan look-backs, TMA fold barriers); synchronous.
inline cudaError_t wait_timeouts(unsigned long long* count) { return total_wait_timeouts(count); }

// A look-back wait that must run out: a two-tile column scanned with the
// ticket counter started at 1, so the block that takes tile 1 waits for a tile
// 0 that no block takes.  The kernel gives up after its bounded polls, writes
// NaN over tile 1 and sets the error word, which is returned in *failed.
inline cudaError_t selftest_wait_timeout(cudaStream_t s, unsigned* failed)
{
  using Op = fold::op_sum<true>;
  using K = scan_tiles<Op, float>;
  const size_t rows = 2 * K::TILE;
  float* buf = nullptr;
  char* scratch = nullptr;
  const size_t head = 256, fbytes = 256, sbytes = align256(2 * carry_bytes<Op, float>());
  cudaError_t e = cudaMalloc(&buf, rows * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&scratch, head + fbytes + 2 * sbytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, rows * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, head + fbytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 1, 1, s);    // ticket = 1
  if (e == cudaSuccess) {
    inner_shape sh;
    sh.rows = rows;
    sh.cols = 1;
    sh.tiles_per_col = 2;
    sh.tiles = 2;
    const float* x = buf;
    float* y = buf;
    int vec = 1;
    unsigned long long* ticket = (unsigned long long*)scratch;
    unsigned* err = (unsigned*)(scratch + 8);
    unsigned* flags = (unsigned*)(scratch + head);
    void* agg = scratch + head + fbytes;
    void* incl = scratch + head + fbytes + sbytes;
    void* args[] = {(void*)&x, (void*)&y, (void*)&sh, (void*)&vec, (void*)&ticket, (void*)&flags, (void*)&agg,
                    (void*)&incl, (void*)&err};
    e = launch_dependent(k_scan_inner<Op, float>, 2, 256, s, args);
    if (e == cudaSuccess) e = cudaMemcpyAsync(failed, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (buf) cudaFree(buf);
  if (scratch) cudaFree(scratch);
  return e;
}

template <class Op, class T, int V>
cudaError_t outer_scan_v(const T* x, T* y, size_t rows, size_t cols, cudaStream_t s)
{
  using S = state_of<Op, T>;
  constexpr size_t ROWS = 256 * (size_t)V;
  outer_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.strips = (rows + ROWS - 1) / ROWS;
  // about two blocks per SM in all; a chunk is a whole number of 8-column groups
  const size_t want = (2 * (size_t)sm_count() + sh.strips - 1) / sh.strips;
  size_t cchunk = (cols + want - 1) / want;
  cchunk = (cchunk + 7) / 8 * 8;
  sh.cchunk = cchunk < 8 ? 8 : cchunk;
  sh.chunks = (cols + sh.cchunk - 1) / sh.cchunk;
  const size_t units = sh.strips * sh.chunks;
  S* totals = nullptr;
  cudaError_t e;
  if (sh.chunks > 1) {
    void* scratch = nullptr;
    if ((e = nt2cuda::stream_scratch(s, units * ROWS * sizeof(S), &scratch, 1)) != cudaSuccess) return e;
    totals = (S*)scratch;
    void* a1[] = {(void*)&x, (void*)&y, (void*)&sh, (void*)&totals};
    if ((e = launch_persistent(k_scan_outer<Op, T, V, false>, units * 256, 256, 2, s, a1)) != cudaSuccess)
      return e;
    void* a2[] = {(void*)&sh, (void*)&totals};
    if ((e = launch_persistent(k_scan_outer_prefix<Op, T, V>, sh.strips * ROWS, 256, 2, s, a2)) != cudaSuccess)
      return e;
  }
  void* a3[] = {(void*)&x, (void*)&y, (void*)&sh, (void*)&totals};
  return launch_persistent(k_scan_outer<Op, T, V, true>, units * 256, 256, 2, s, a3);
}

// The TMA-staged row scan (k_scan_outer_tma): one block per strip of
// 128 bytes of rows walking all columns.  cudaErrorNotSupported, before
// anything is launched, when the tensor maps cannot be made.
template <class Op, class T>
cudaError_t outer_scan_staged(const T* x, T* y, size_t rows, size_t cols, cudaStream_t s)
{
  constexpr int BR = outer_tma_rows<T>(), BC = kOuterTmaCols, STAGES = 6;
  PFN_cuTensorMapEncodeTiled_v12000 encode = tma::tensor_map_encoder();
  if (!encode) return cudaErrorNotSupported;
  CUtensorMap xmap, ymap;
  const cuuint64_t gdim[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  const cuuint64_t gstride[1] = {(cuuint64_t)(rows * sizeof(T))};
  const cuuint32_t box[2] = {(cuuint32_t)BR, (cuuint32_t)BC};
  const cuuint32_t estride[2] = {1, 1};
  const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  if (encode(&xmap, dt, 2, (void*)x, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
      encode(&ymap, dt, 2, (void*)y, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorNotSupported;
  outer_tma_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.strips = (rows + BR - 1) / BR;
  sh.ctiles = (cols + BC - 1) / BC;
  sh.wait_rounds = tma::kMaxRounds;
  auto k = k_scan_outer_tma<Op, T, STAGES>;
  const int smem = STAGES * BR * BC * (int)sizeof(T);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&xmap, (void*)&ymap, (void*)&sh};
  return launch_dependent(k, sh.strips, 256, s, args, smem);
}

template <class Op, class T>
cudaError_t outer_scan(const T* x, T* y, size_t rows, size_t cols, cudaStream_t s)
{
  if (!rows || !cols) return cudaSuccess;
  constexpr int V = 16 / (int)sizeof(T);
  // at least one strip of 128 bytes of rows per SM: the staged single pass
  if ((((uintptr_t)x | (uintptr_t)y) & 15u) == 0 && rows % V == 0 && rows < ((size_t)1 << 31) &&
      cols < ((size_t)1 << 31) && rows / (size_t)outer_tma_rows<T>() >= (size_t)sm_count()) {
    const cudaError_t e = outer_scan_staged<Op, T>(x, y, rows, cols, s);
    if (e != cudaErrorNotSupported) return e;
  }
  if ((((uintptr_t)x | (uintptr_t)y) & 15u) == 0 && rows % V == 0) return outer_scan_v<Op, T, V>(x, y, rows, cols, s);
  return outer_scan_v<Op, T, 1>(x, y, rows, cols, s);
}

template <class Op, class T>
cudaError_t scan_dim(const T* x, T* y, size_t rows, size_t cols, int dim, cudaStream_t s)
{
  return dim == 1 ? inner_scan<Op, T>(x, y, rows, cols, s) : outer_scan<Op, T>(x, y, rows, cols, s);
}

}  // namespace scan
}  // namespace nt2cuda
