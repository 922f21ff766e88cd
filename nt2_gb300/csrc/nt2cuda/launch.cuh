// nt2cuda/launch.cuh -- host side of the fused transform: picks the kernel
// variant for a lowered statement and sizes its persistent grid.
//
// This is the GB300 replacement for NT2's transform spawner
// (modules/arch/shared_memory/include/nt2/core/functions/shared_memory/transform.hpp:26-50,
//  modules/arch/openmp/include/nt2/sdk/openmp/spawner/transform.hpp:30-74): instead of
// chunking [0,n) over OpenMP threads in L2-sized grains, one launch covers the
// whole range with a grid of (SM count x resident blocks per SM).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "expr.cuh"
#include "tuning.cuh"

namespace nt2cuda {

// ------------------------------------------------- pointer enumeration
struct ptr_span { const void* p; size_t bytes; bool out; int assign; };

template <class T, class F> inline void visit_expr(const scal<T>&, F&&, int) {}
template <class T, class F> inline void visit_expr(const term<T>& t, F&& f, int a)
{ f(ptr_span{t.p, sizeof(T), false, a}); }
template <class Tag, class... C, class F> inline void visit_expr(const node<Tag, C...>& n, F&& f, int a);
template <class Tag, class A, class F> inline void visit_node(const node<Tag, A>& n, F&& f, int a)
{ visit_expr(n.a, f, a); }
template <class Tag, class A, class B, class F> inline void visit_node(const node<Tag, A, B>& n, F&& f, int a)
{ visit_expr(n.a, f, a); visit_expr(n.b, f, a); }
template <class Tag, class A, class B, class C, class F> inline void visit_node(const node<Tag, A, B, C>& n, F&& f, int a)
{ visit_expr(n.a, f, a); visit_expr(n.b, f, a); visit_expr(n.c, f, a); }
template <class Tag, class... C, class F> inline void visit_expr(const node<Tag, C...>& n, F&& f, int a)
{ visit_node(n, f, a); }

template <class F> inline void visit_prog(const prog<>&, F&&, int) {}
template <class T, class E, class... As, class F>
inline void visit_prog(const prog<assign<T, E>, As...>& p, F&& f, int a = 0)
{
  f(ptr_span{p.head.out, sizeof(T), true, a});
  visit_expr(p.head.e, f, a);
  visit_prog(p.tail, f, a + 1);
}

enum class alias_kind { none, bad };

// Classify how the inputs of a statement alias its outputs over n elements.
// An input that is exactly one of the statement's outputs is fine: NT2
// evaluates every right-hand side of a statement (all members of a tie())
// at an index before it stores any output
// (modules/core/container/table/include/nt2/core/functions/expr/tie.hpp:70-95),
// and the kernel does the same, each element read by the thread that later
// writes it.  Partial overlaps, and one table bound to two outputs, are
// rejected.
template <class P> inline alias_kind classify_alias(const P& p, size_t n)
{
  ptr_span spans[64]; int ns = 0;
  bool overflow = false;
  visit_prog(p, [&](ptr_span s) { if (ns < 64) spans[ns++] = s; else overflow = true; });
  if (overflow) return alias_kind::bad;
  for (int i = 0; i < ns; ++i) {
    if (!spans[i].out) continue;
    const char* o0 = (const char*)spans[i].p; const char* o1 = o0 + n * spans[i].bytes;
    for (int j = 0; j < ns; ++j) {
      if (i == j) continue;
      const char* a0 = (const char*)spans[j].p; const char* a1 = a0 + n * spans[j].bytes;
      if (a1 <= o0 || o1 <= a0) continue;                      // disjoint
      if (a0 != o0 || spans[j].bytes != spans[i].bytes) return alias_kind::bad;
      if (spans[j].out) return alias_kind::bad;                // two outputs on one table
    }
  }
  return alias_kind::none;
}

template <class P> inline bool all_aligned(const P& p, unsigned align)
{
  bool ok = true;
  visit_prog(p, [&](ptr_span s) { if (((uintptr_t)s.p) % align) ok = false; });
  return ok;
}

// ----------------------------------------------------------- launching
inline int sm_count()
{
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

template <class K> inline int resident_blocks(K kernel, int block)
{
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, block, 0) != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

// Launch as a programmatic dependent of the previous kernel on the stream:
// the grid may be scheduled while its predecessor finishes, and waits in
// pdl_begin() until the predecessor has completed and its writes are visible.
// Every kernel launched this way starts with pdl_begin().
template <class K>
inline cudaError_t launch_dependent(K kernel, size_t grid, int block, cudaStream_t s, void** args,
                                    size_t smem = 0)
{
  if (grid < 1) grid = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, (const void*)kernel, args);
}

template <class K>
inline cudaError_t launch_persistent(K kernel, size_t work_items, int block, int waves,
                                     cudaStream_t s, void** args)
{
  int per_sm = resident_blocks(kernel, block);
  size_t full = (size_t)sm_count() * (size_t)per_sm * (size_t)(waves > 0 ? waves : 1);
  size_t need = (work_items + (size_t)block - 1) / (size_t)block;
  size_t grid = need < full ? need : full;
  return launch_dependent(kernel, grid, block, s, args);
}

// Launch with an explicit grid (at least one block).
template <class K>
inline cudaError_t launch_grid(K kernel, size_t grid, int block, cudaStream_t s, void** args)
{
  return launch_dependent(kernel, grid, block, s, args);
}

// Evaluate statement p over [0,n).  Returns cudaErrorInvalidValue when the
// statement's tables partially overlap.  `def` is used when the tuning table
// has no entry for tune_key at this size.
template <bool F, class P>
inline cudaError_t transform(const P& p, size_t n, cudaStream_t s, const char* tune_key = nullptr,
                             tuning::params def = tuning::params{})
{
  if (n == 0) return cudaSuccess;
  alias_kind ak = classify_alias(p, n);
  if (ak == alias_kind::bad) return cudaErrorInvalidValue;
  constexpr int V = base_lanes<P>::value;
  // statements with three or more long functors: one group per thread per trip
  if (prog_heavy<P>::value >= 3 && def.unroll == tuning::params{}.unroll) def.unroll = 1;
  const tuning::params tp = tuning::lookup(tune_key, n, def);
  const int U = tp.unroll, W = tp.waves;
  P pc = p;
  size_t nn = n;
  void* args[] = {&pc, &nn};
  const bool vec = all_aligned(p, 16u);
  if (!vec) return launch_persistent(k_transform<F, 1, 1, P>, n, 256, W, s, args);
  const size_t groups = n / V;
  switch (U) {
    case 1: return launch_persistent(k_transform<F, V, 1, P>, groups, 256, W, s, args);
    case 4: return launch_persistent(k_transform<F, V, 4, P>, groups, 256, W, s, args);
    default: return launch_persistent(k_transform<F, V, 2, P>, groups, 256, W, s, args);
  }
}

}  // namespace nt2cuda
