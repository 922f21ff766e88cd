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
#include "fold_tma.cuh"
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>

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

// Which kernels serve the folds of a table or of a product of two tables:
//   0 (auto): TMA-staged for long columns (inner_fold, rows >= 2^16), the
//             register-pipelined kernels otherwise;
//   1 (simt): always the register-pipelined kernels;
//   2 (tma):  TMA-staged wherever the tables allow it (16-byte aligned, whole
//             vectors long; outer_fold from 256 rows).
// The initial value comes from NT2CUDA_FOLD_PATH ("auto", "simt", "tma").
inline std::atomic<int>& fold_path()
{
  static std::atomic<int> p([] {
    const char* e = getenv("NT2CUDA_FOLD_PATH");
    if (e && !strcmp(e, "simt")) return 1;
    if (e && !strcmp(e, "tma")) return 2;
    return 0;
  }());
  return p;
}

template <class T> struct tma_terms { static constexpr int n = 0; };
template <class T> struct tma_terms<term<T>> { static constexpr int n = 1; };
template <class T> struct tma_terms<node<tag::multiplies_, term<T>, term<T>>> { static constexpr int n = 2; };

template <class T> inline const T* first_term(const term<T>& t) { return t.p; }
template <class T> inline const T* first_term(const node<tag::multiplies_, term<T>, term<T>>& n) { return n.a.p; }
template <class T> inline const T* second_term(const term<T>&) { return nullptr; }
template <class T> inline const T* second_term(const node<tag::multiplies_, term<T>, term<T>>& n) { return n.b.p; }

// Loads in flight per lane in the register-pipelined kernels: 16 (8 left the
// 134 MB folds at 71% of the copy peak, 16 reaches 75-77%, 32 adds nothing),
// or 8 for var/stdev, whose block updates (add_block) hold the loaded values
// until the block's mean is known.
template <class Op> struct fold_unroll { static constexpr int value = 16; };
template <bool W1, bool SD> struct fold_unroll<op_moments<W1, SD>> { static constexpr int value = 8; };
// outer_fold keeps V rows' states per lane: var/stdev there take 4 columns a trip
template <class Op> struct outer_unroll { static constexpr int value = fold_unroll<Op>::value; };
template <bool W1, bool SD> struct outer_unroll<op_moments<W1, SD>> { static constexpr int value = 4; };

template <class Op, class T> cudaError_t fold_empty(out_of<Op, T>* out, size_t count, cudaStream_t s)
{
  void* args[] = {&out, &count};
  return launch_persistent(k_fold_empty<Op, T>, count, 256, 1, s, args);
}

// inner_fold with operation Op (op_sum<COMP>, op_val, op_logic, op_moments).
template <class Op, class T, class E>
cudaError_t inner_fold(const E& e, size_t rows, size_t cols, out_of<Op, T>* out, cudaStream_t s)
{
  using S = state_of<Op, T>;
  if constexpr (tma_terms<E>::n > 0) {
    constexpr size_t VV = 16 / sizeof(T);
    // auto: long columns only; a short column's tiles are too few to amortise the block barriers
    const int path = fold_path().load(std::memory_order_relaxed);
    const size_t min_rows = path == 2 ? 32 : ((size_t)1 << 16);
    if (path != 1 && rows >= min_rows && cols > 0 && out && rows % VV == 0 && expr_aligned(e) &&
        std::is_same<typename value_of<E>::type, T>::value)
      return inner_fold_tma<Op, T>(first_term(e), second_term(e), rows, cols, out, s);
  }
  if (cols == 0) return cudaSuccess;
  if (!out) return cudaErrorInvalidValue;
  if (rows == 0) return fold_empty<Op, T>(out, cols, s);
  if (rows < 32) {
    size_t ee = cols;
    E ec = e;
    out_of<Op, T>* o = out;
    void* args[] = {&ec, &rows, &ee, &o};
    return (launch_persistent(k_inner_short<Op, T, E>, cols, 256, 4, s, args));
  }
  constexpr int VV = 16 / (int)sizeof(T);
  const bool vec = expr_aligned(e) && rows % VV == 0;
  inner_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.seg = inner_seg<T>();
  sh.splits = (rows + sh.seg - 1) / sh.seg;
  S* partials = nullptr;
  unsigned* counters = nullptr;
  if (sh.splits > 1) {
    void* p = nullptr;
    cudaError_t st = fold_scratch(s, cols, cols * sh.splits, sizeof(S), &counters, &p);
    if (st != cudaSuccess) return st;
    partials = (S*)p;
  }
  const size_t units = cols * sh.splits;
  E ec = e;
  out_of<Op, T>* o = out;
  void* args[] = {&ec, &sh, &o, &partials, &counters};
  // launch_persistent counts threads; a unit is one warp
  if (vec) return (launch_persistent(k_inner<Op, VV, fold_unroll<Op>::value, T, E>, units * 32, 128, 4, s, args));
  return (launch_persistent(k_inner<Op, 1, 4, T, E>, units * 32, 256, 4, s, args));
}

template <class Op, class T, class E>
cudaError_t outer_fold(const E& e, size_t rows, size_t cols, out_of<Op, T>* out, cudaStream_t s)
{
  using S = state_of<Op, T>;
  if constexpr (tma_terms<E>::n == 1) {
    constexpr size_t VV = 16 / sizeof(T);
    if (fold_path().load(std::memory_order_relaxed) == 2 && rows >= 256 && cols > 0 && out && rows % VV == 0 &&
        expr_aligned(e) && rows < ((size_t)1 << 31) && cols < ((size_t)1 << 31)) {
      cudaError_t r = outer_fold_tma<Op, T>(first_term(e), rows, cols, out, s);
      if (r != cudaErrorNotSupported) return r;
    }
  }
  if (rows == 0) return cudaSuccess;
  if (!out) return cudaErrorInvalidValue;
  if (cols == 0) return fold_empty<Op, T>(out, rows, s);
  constexpr int VV = 16 / (int)sizeof(T);
  const bool vec = expr_aligned(e) && rows % VV == 0;
  const int V = vec ? VV : 1;
  const size_t STRIP = (size_t)32 * V;
  outer_shape sh;
  sh.rows = rows;
  sh.cols = cols;
  sh.strips = (rows + STRIP - 1) / STRIP;
  // about 512 blocks in all, so the grid fits in one wave of resident blocks
  // (the split depends only on the shape, so results stay reproducible)
  {
    const size_t want_splits = (512 + sh.strips - 1) / sh.strips;
    size_t cchunk = (cols + want_splits - 1) / want_splits;
    cchunk = (cchunk + 63) / 64 * 64;
    sh.cchunk = cchunk < 64 ? 64 : cchunk;
  }
  sh.splits = (cols + sh.cchunk - 1) / sh.cchunk;
  S* partials = nullptr;
  unsigned* counters = nullptr;
  if (sh.splits > 1) {
    void* p = nullptr;
    cudaError_t st = fold_scratch(s, sh.strips, sh.strips * sh.splits * STRIP, sizeof(S), &counters, &p);
    if (st != cudaSuccess) return st;
    partials = (S*)p;
  }
  const size_t units = sh.strips * sh.splits;
  E ec = e;
  out_of<Op, T>* o = out;
  void* args[] = {&ec, &sh, &o, &partials, &counters};
  if (vec) return (launch_persistent(k_outer<Op, VV, outer_unroll<Op>::value, T, E>, units * 256, 256, 4, s, args));
  return (launch_persistent(k_outer<Op, 1, 4, T, E>, units * 256, 256, 4, s, args));
}

}  // namespace fold
}  // namespace nt2cuda

