// nt2cuda/fold_launch.cuh -- host launchers of the inner_fold and outer_fold
// kernels for any elementwise expression E (globalsum(X*Y) is
// inner_fold(node<multiplies_, term, term>, n, 1)).
// The NT2 overloads they replace are
// modules/arch/shared_memory/include/nt2/core/functions/shared_memory/inner_fold.hpp:24-63 and
// .../shared_memory/outer_fold.hpp:22-51.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "expr.cuh"
#include "fold.cuh"
#include "launch.cuh"
#include "scratch.cuh"

namespace nt2cuda {
namespace fold {

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class E> bool expr_aligned(const E& e)
{
  bool ok = true;
  visit_expr(e, [&](ptr_span s) { if (((uintptr_t)s.p) & 15u) ok = false; }, 0);
  return ok;
}

// Segment length of one warp's share of a column: 128 vector groups per lane.
template <class T> constexpr size_t inner_seg() { return (size_t)32 * (16 / sizeof(T)) * 128; }

template <bool COMP, class T, class E>
cudaError_t inner_fold(const E& e, size_t rows, size_t cols, T* out, cudaStream_t s)
{
  if (cols == 0) return cudaSuccess;
  if (!out) return cudaErrorInvalidValue;
  if (rows == 0) return (cudaMemsetAsync(out, 0, cols * sizeof(T), s));
  if (rows < 32) {
    size_t ee = cols;
    E ec = e;
    T* o = out;
    void* args[] = {&ec, &rows, &ee, &o};
    return (launch_persistent(k_inner_short<COMP, T, E>, cols, 256, 4, s, args));
  }
  constexpr int VV = 16 / (int)sizeof(T);
  const bool vec = expr_aligned(e) && rows % VV == 0;
  inner_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.seg = inner_seg<T>();
  sh.splits = (rows + sh.seg - 1) / sh.seg;
  acc<T>* partials = nullptr;
  unsigned* counters = nullptr;
  if (sh.splits > 1) {
    size_t cbytes = round_up(cols * sizeof(unsigned), 256);
    size_t pbytes = cols * sh.splits * sizeof(acc<T>);
    void* scratch = nullptr;
    cudaError_t st = stream_scratch(s, cbytes + pbytes, &scratch);
    if (st != cudaSuccess) return st;
    counters = (unsigned*)scratch;
    partials = (acc<T>*)((char*)scratch + cbytes);
  }
  const size_t units = cols * sh.splits;
  E ec = e;
  T* o = out;
  void* args[] = {&ec, &sh, &o, &partials, &counters};
  // launch_persistent counts threads; a unit is one warp
  if (vec) return (launch_persistent(k_inner<COMP, VV, 4, T, E>, units * 32, 256, 4, s, args));
  return (launch_persistent(k_inner<COMP, 1, 4, T, E>, units * 32, 256, 4, s, args));
}

template <bool COMP, class T, class E>
cudaError_t outer_fold(const E& e, size_t rows, size_t cols, T* out, cudaStream_t s)
{
  if (rows == 0) return cudaSuccess;
  if (!out) return cudaErrorInvalidValue;
  if (cols == 0) return (cudaMemsetAsync(out, 0, rows * sizeof(T), s));
  constexpr int VV = 16 / (int)sizeof(T);
  const bool vec = expr_aligned(e) && rows % VV == 0;
  const int V = vec ? VV : 1;
  const size_t STRIP = (size_t)32 * V;
  outer_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.cchunk = 256;
  sh.splits = (cols + sh.cchunk - 1) / sh.cchunk;
  sh.strips = (rows + STRIP - 1) / STRIP;
  acc<T>* partials = nullptr;
  unsigned* counters = nullptr;
  if (sh.splits > 1) {
    size_t cbytes = round_up(sh.strips * sizeof(unsigned), 256);
    size_t pbytes = sh.strips * sh.splits * STRIP * sizeof(acc<T>);
    void* scratch = nullptr;
    cudaError_t st = stream_scratch(s, cbytes + pbytes, &scratch);
    if (st != cudaSuccess) return st;
    counters = (unsigned*)scratch;
    partials = (acc<T>*)((char*)scratch + cbytes);
  }
  const size_t units = sh.strips * sh.splits;
  E ec = e;
  T* o = out;
  void* args[] = {&ec, &sh, &o, &partials, &counters};
  if (vec) return (launch_persistent(k_outer<COMP, VV, 4, T, E>, units * 256, 256, 4, s, args));
  return (launch_persistent(k_outer<COMP, 1, 4, T, E>, units * 256, 256, 4, s, args));
}

}  // namespace fold
}  // namespace nt2cuda

