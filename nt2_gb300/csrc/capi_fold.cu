// capi_fold.cu -- C-ABI entry points for the inner_fold / outer_fold site
// overloads: globalsum, dot (globalsum of X*Y), sum(A,1) and sum(A,2).
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/fold.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;
using nt2cuda::fold::acc;

namespace {

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
nt2cuda_status inner_fold(const E& e, size_t rows, size_t cols, T* out, cudaStream_t s)
{
  if (cols == 0) return NT2CUDA_OK;
  if (!out) return NT2CUDA_ERR_ARG;
  if (rows == 0) return from_cuda(cudaMemsetAsync(out, 0, cols * sizeof(T), s));
  if (rows < 32) {
    size_t ee = cols;
    E ec = e;
    T* o = out;
    void* args[] = {&ec, &rows, &ee, &o};
    return launch_status(launch_persistent(fold::k_inner_short<COMP, T, E>, cols, 256, 4, s, args));
  }
  constexpr int VV = 16 / (int)sizeof(T);
  const bool vec = expr_aligned(e) && rows % VV == 0;
  fold::inner_shape sh;
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
    nt2cuda_status st = stream_scratch(s, cbytes + pbytes, &scratch);
    if (st != NT2CUDA_OK) return st;
    counters = (unsigned*)scratch;
    partials = (acc<T>*)((char*)scratch + cbytes);
  }
  const size_t units = cols * sh.splits;
  E ec = e;
  T* o = out;
  void* args[] = {&ec, &sh, &o, &partials, &counters};
  // launch_persistent counts threads; a unit is one warp
  if (vec) return launch_status(launch_persistent(fold::k_inner<COMP, VV, 4, T, E>, units * 32, 256, 4, s, args));
  return launch_status(launch_persistent(fold::k_inner<COMP, 1, 4, T, E>, units * 32, 256, 4, s, args));
}

template <bool COMP, class T, class E>
nt2cuda_status outer_fold(const E& e, size_t rows, size_t cols, T* out, cudaStream_t s)
{
  if (rows == 0) return NT2CUDA_OK;
  if (!out) return NT2CUDA_ERR_ARG;
  if (cols == 0) return from_cuda(cudaMemsetAsync(out, 0, rows * sizeof(T), s));
  constexpr int VV = 16 / (int)sizeof(T);
  const bool vec = expr_aligned(e) && rows % VV == 0;
  const int V = vec ? VV : 1;
  const size_t STRIP = (size_t)32 * V;
  fold::outer_shape sh;
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
    nt2cuda_status st = stream_scratch(s, cbytes + pbytes, &scratch);
    if (st != NT2CUDA_OK) return st;
    counters = (unsigned*)scratch;
    partials = (acc<T>*)((char*)scratch + cbytes);
  }
  const size_t units = sh.strips * sh.splits;
  E ec = e;
  T* o = out;
  void* args[] = {&ec, &sh, &o, &partials, &counters};
  if (vec) return launch_status(launch_persistent(fold::k_outer<COMP, VV, 4, T, E>, units * 256, 256, 4, s, args));
  return launch_status(launch_persistent(fold::k_outer<COMP, 1, 4, T, E>, units * 256, 256, 4, s, args));
}

}  // namespace

extern "C" {

nt2cuda_status nt2cuda_globalsum_f32(const float* x, size_t n, float* out, int compensated, nt2cuda_stream s)
{
  if (n && !x) return NT2CUDA_ERR_ARG;
  term<float> e{x};
  return compensated ? inner_fold<true, float>(e, n, 1, out, as_stream(s))
                     : inner_fold<false, float>(e, n, 1, out, as_stream(s));
}

nt2cuda_status nt2cuda_dot_f32(const float* x, const float* y, size_t n, float* out, int compensated,
                               nt2cuda_stream s)
{
  if (n && (!x || !y)) return NT2CUDA_ERR_ARG;
  node<tag::multiplies_, term<float>, term<float>> e{term<float>{x}, term<float>{y}};
  return compensated ? inner_fold<true, float>(e, n, 1, out, as_stream(s))
                     : inner_fold<false, float>(e, n, 1, out, as_stream(s));
}

nt2cuda_status nt2cuda_globalsum_f64(const double* x, size_t n, double* out, nt2cuda_stream s)
{
  if (n && !x) return NT2CUDA_ERR_ARG;
  return inner_fold<false, double>(term<double>{x}, n, 1, out, as_stream(s));
}

nt2cuda_status nt2cuda_dot_f64(const double* x, const double* y, size_t n, double* out, nt2cuda_stream s)
{
  if (n && (!x || !y)) return NT2CUDA_ERR_ARG;
  node<tag::multiplies_, term<double>, term<double>> e{term<double>{x}, term<double>{y}};
  return inner_fold<false, double>(e, n, 1, out, as_stream(s));
}

nt2cuda_status nt2cuda_sum_inner_f32(const float* A, size_t rows, size_t cols, float* out, int compensated,
                                     nt2cuda_stream s)
{
  if (rows && cols && !A) return NT2CUDA_ERR_ARG;
  term<float> e{A};
  return compensated ? inner_fold<true, float>(e, rows, cols, out, as_stream(s))
                     : inner_fold<false, float>(e, rows, cols, out, as_stream(s));
}

nt2cuda_status nt2cuda_sum_inner_f64(const double* A, size_t rows, size_t cols, double* out, nt2cuda_stream s)
{
  if (rows && cols && !A) return NT2CUDA_ERR_ARG;
  return inner_fold<false, double>(term<double>{A}, rows, cols, out, as_stream(s));
}

nt2cuda_status nt2cuda_sum_outer_f32(const float* A, size_t rows, size_t cols, float* out, int compensated,
                                     nt2cuda_stream s)
{
  if (rows && cols && !A) return NT2CUDA_ERR_ARG;
  term<float> e{A};
  return compensated ? outer_fold<true, float>(e, rows, cols, out, as_stream(s))
                     : outer_fold<false, float>(e, rows, cols, out, as_stream(s));
}

nt2cuda_status nt2cuda_sum_outer_f64(const double* A, size_t rows, size_t cols, double* out, nt2cuda_stream s)
{
  if (rows && cols && !A) return NT2CUDA_ERR_ARG;
  return outer_fold<false, double>(term<double>{A}, rows, cols, out, as_stream(s));
}

}  // extern "C"
