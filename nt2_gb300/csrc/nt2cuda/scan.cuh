// nt2cuda/scan.cuh -- inner_scan and outer_scan: cumsum, cumprod, cummax and
// cummin of a column-major table along dimension 1 or 2.
//
// NT2 evaluates a cumulative function through inner_scan (the scanned
// dimension is the first non-singleton one) or outer_scan
// (modules/core/swar/include/nt2/dsl/functions/cumulative/run.hpp:27-75); both
// fold `summary = bop(summary, x)` in index order and store every summary
// (modules/core/swar/include/nt2/core/functions/details/scan_step.hpp:32-44);
// the OpenMP spawner scans blocks of `grain` elements and rescans each block
// from the bop of the earlier blocks' summaries
// (modules/arch/openmp/include/nt2/sdk/openmp/spawner/scan.hpp:32-121).
//
// inner_scan here is one launch.  A column of at most 32 KB is one tile, read
// once into registers and scanned in place (k_scan_inner_1p).  Longer columns
// are cut into 64 KB tiles chained by a decoupled look-back (k_scan_inner):
// each tile's aggregate is published, its prefix formed from the
// predecessors' published aggregates and inclusive prefixes, and the tile
// rescanned from that prefix.  The prefix of tile t is defined as the left
// fold I(t-1) = bop(I(t-2), A(t-1)) of the tile aggregates; for FP32 sums the
// carries are exact integers and for max/min the operation is exact, so any
// window of predecessors may be combined in any order; for the other
// operations the look-back folds at most 31 aggregates forward from the
// nearest published I(p).  Either way the prefix is the same whatever the
// timing, so results are bitwise reproducible.  Tiles are handed out by an
// atomic ticket, so a tile only ever waits for tiles that running blocks
// already hold; every wait is bounded, and a tile whose wait runs out writes
// NaN and passes a failure flag on instead of a prefix.
//
// outer_scan of a table with at least one 128-byte strip of rows per SM is one
// pass (k_scan_outer_tma): each block walks the columns of its strip in order,
// tiles streamed through shared memory by TMA, the rows' running values kept
// on chip.  Narrower tables run in two launches: the per-row totals of column
// chunks, then each chunk rescanned from the left fold of the earlier chunks'
// totals.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fold.cuh"
#include "memory.cuh"
#include "tma.cuh"

namespace nt2cuda {
namespace scan {

using fold::state_of;

constexpr int kWarps = 8;
// A thread owns 8 consecutive 16-byte chunks (32 floats or 16 doubles) of its
// warp's span; a tile is 256 threads x 128 bytes = 32 KB.
template <class T> __host__ __device__ constexpr int chunk_elems() { return 16 / (int)sizeof(T); }
template <class T> __host__ __device__ constexpr int thread_elems() { return 8 * chunk_elems<T>(); }
template <class T> __host__ __device__ constexpr int tile() { return kWarps * 32 * thread_elems<T>(); }
// Bounded polls of one flag: with the 64 ns sleeps and the load latency a
// wait gives up after well under a second; a tile's predecessors are held by
// running blocks that never wait on it, so a wait that runs out means a fault.
constexpr unsigned kSpinMax = 1u << 20;

// Look-back waits that ran out, over the life of the process (read by
// nt2cuda_wait_timeouts); a tile whose wait runs out writes NaN and passes a
// failure flag to its successors.
static __device__ unsigned long long g_wait_timeouts = 0;

enum : unsigned { F_NONE = 0, F_AGG = 1, F_INCL = 2, F_FAIL = 3 };

struct inner_shape {
  size_t rows, cols, tiles_per_col, tiles;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p)
{
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// with the relaxed loads before it that saw a released flag: acquire
__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <class T> __device__ __forceinline__ T nan_value()
{
  if constexpr (sizeof(T) == 4) return __int_as_float(0x7fc00000);
  else return __longlong_as_double(0x7ff8000000000000ll);
}

// Bounded wait for a published flag; F_NONE when the wait ran out.
__device__ __forceinline__ unsigned wait_flag(const unsigned* p)
{
  unsigned f = ld_acquire(p);
  for (unsigned it = 0; f == F_NONE && it < kSpinMax; ++it) {
    __nanosleep(64);
    f = ld_acquire(p);
  }
  return f;
}

// Shared-memory layout of one warp's span: lane l's 8 chunks at 16-byte slots
// l*9 .. l*9+7 (one slot of padding per lane).  The coalesced load of chunk
// q = 32*i + l (lane l, load i) lands in owner lane q/8, slot q%8; both that
// store and the owner's own reads touch 8 distinct 16-byte bank groups per
// quarter-warp, so neither conflicts.
__device__ __forceinline__ int slot_of(int owner, int c) { return owner * 9 + c; }

// ------------------------------------------------------ exact carries
// Tile prefixes of FP32 sums travel as exact 320-bit two's complement fixed
// point numbers (least significant bit 2^-160, so every finite float and any
// sum of up to 2^31 of them is represented exactly).  Integer addition is
// associative, so the look-back may add up any window of predecessors in any
// order -- here a warp-wide tree -- and the prefix is the same bits whatever
// the timing.  Non-finite aggregates are carried beside the integer as a float.
struct xsum {
  unsigned long long w[5];
  float special;        // sum of the non-finite aggregates (0 when there are none)
  unsigned has_special;
};

__device__ __forceinline__ xsum xzero()
{
  xsum r;
#pragma unroll
  for (int i = 0; i < 5; ++i) r.w[i] = 0ull;
  r.special = 0.f;
  r.has_special = 0u;
  return r;
}

__device__ __forceinline__ void xadd_into(xsum& a, const xsum& b)
{
  unsigned long long carry = 0ull;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const unsigned long long s1 = a.w[i] + b.w[i];
    const unsigned long long c1 = s1 < a.w[i] ? 1ull : 0ull;
    const unsigned long long s2 = s1 + carry;
    const unsigned long long c2 = s2 < s1 ? 1ull : 0ull;
    a.w[i] = s2;
    carry = c1 + c2;
  }
  if (b.has_special) {
    a.special = a.has_special ? a.special + b.special : b.special;
    a.has_special = 1u;
  }
}

// Add the float f exactly.
__device__ __forceinline__ void xadd_float(xsum& a, float f)
{
  if (f == 0.f) return;
  if (!isfinite(f)) {
    a.special = a.has_special ? a.special + f : f;
    a.has_special = 1u;
    return;
  }
  const unsigned u = __float_as_uint(f);
  const int be = (int)((u >> 23) & 0xffu);
  const unsigned long long m = be ? (unsigned long long)((u & 0x7fffffu) | 0x800000u) : (unsigned long long)(u & 0x7fffffu);
  const int sh = (be ? be - 127 : -126) + 137;   // bit position of m's lowest bit (value m * 2^(e-23), lsb 2^-160)
  xsum b = xzero();
  const int li = sh >> 6, bi = sh & 63;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    unsigned long long lo = (i == li) ? (m << bi) : 0ull;
    unsigned long long hi = (i == li + 1 && bi) ? (m >> (64 - bi)) : 0ull;
    b.w[i] = lo | hi;
  }
  if (u >> 31) {   // two's complement negation
    unsigned long long carry = 1ull;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const unsigned long long n = ~b.w[i] + carry;
      carry = (carry && n == 0ull) ? 1ull : 0ull;
      b.w[i] = n;
    }
  }
  xadd_into(a, b);
}

// A float pair (s, c) for the exact value, in integer arithmetic (a fixed
// function of the bits, so equal sums give equal pairs): s is the value
// rounded to nearest even (the few values below the smallest subnormal read as
// zero), c the rest (the 128 bits of the value from its leading one, minus s)
// rounded from its leading 64 bits.
__device__ __forceinline__ fold::acc<float> xto_pair(const xsum& x)
{
  if (x.has_special) return fold::acc<float>{x.special, 0.f};
  unsigned long long w[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) w[i] = x.w[i];
  const bool neg = (w[4] >> 63) != 0ull;
  if (neg) {
    unsigned long long carry = 1ull;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const unsigned long long n = ~w[i] + carry;
      carry = (carry && n == 0ull) ? 1ull : 0ull;
      w[i] = n;
    }
  }
  int top = -1;
#pragma unroll
  for (int i = 4; i >= 0; --i)
    if (top < 0 && w[i]) top = i;
  if (top < 0) return fold::acc<float>{0.f, 0.f};
  unsigned long long hi = 0ull, mid = 0ull;
  bool low = false;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    if (i == top) hi = w[i];
    if (i == top - 1) mid = w[i];
    if (i < top - 1 && w[i]) low = true;
  }
  const int n = __clzll((long long)hi);
  const unsigned long long T = n ? (hi << n) | (mid >> (64 - n)) : hi;   // leading one at bit 63
  const unsigned long long R = mid << n;
  const int E = 64 * top + 63 - n - 160;                                 // T's leading one is 2^E
  if (E < -149) return fold::acc<float>{0.f, 0.f};
  const int k = (E + 150 < 24) ? E + 150 : 24;                           // bits s keeps
  unsigned long long m = T >> (64 - k);
  const unsigned long long rest = T << k;
  const bool up = (rest >> 63) != 0ull && ((rest << 1) != 0ull || R != 0ull || low || (m & 1ull));
  if (up) ++m;
  float s = ldexpf((float)m, E - k + 1);
  float c = 0.f;
  if (!isinf(s)) {
    const unsigned __int128 X = ((unsigned __int128)T << 64) | R;
    const unsigned __int128 M = (unsigned __int128)m << (128 - k);      // wraps to 0 when m = 2^k: M - X is then 2^128 - X
    const unsigned __int128 d = up ? M - X : X - M;                       // |value - s| in units of 2^(E-127)
    const unsigned long long dh = (unsigned long long)(d >> 64), dl = (unsigned long long)d;
    if (dh | dl) {
      const int rn = dh ? __clzll((long long)dh) : 64 + __clzll((long long)dl);
      const unsigned long long top64 = (unsigned long long)((d << rn) >> 64);
      c = ldexpf(__ull2float_rn(top64), E - 127 + 64 - rn);
      if (up) c = -c;
    }
  }
  if (neg) {
    s = -s;
    c = -c;
  }
  return fold::acc<float>{s, c};
}

__device__ __forceinline__ xsum xshfl_xor(const xsum& a, int off)
{
  xsum r;
#pragma unroll
  for (int i = 0; i < 5; ++i) r.w[i] = __shfl_xor_sync(0xffffffffu, a.w[i], off);
  r.special = __shfl_xor_sync(0xffffffffu, a.special, off);
  r.has_special = __shfl_xor_sync(0xffffffffu, a.has_special, off);
  return r;
}

// Sum over the warp; exact, so the combination order does not matter.
__device__ __forceinline__ xsum xwarp_sum(xsum a)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const xsum o = xshfl_xor(a, off);
    xadd_into(a, o);
  }
  return a;
}

__device__ __forceinline__ void xstore(xsum* p, const xsum& v) { *p = v; }
__device__ __forceinline__ xsum xload(const xsum* p)
{
  xsum r;
#pragma unroll
  for (int i = 0; i < 5; ++i) r.w[i] = __ldcg(&p->w[i]);
  r.special = __ldcg(&p->special);
  r.has_special = __ldcg(&p->has_special);
  return r;
}

// How a tile's look-back combines its predecessors:
//   exact  (FP32 sums): exact integer carries, any window, warp-tree sums;
//   tree   (max, min):  the operation is exact, any window, warp-tree merges;
//   serial (the rest):  at most 31 aggregates folded in index order from the
//                       nearest inclusive prefix.
enum carry_kind { CARRY_SERIAL = 0, CARRY_EXACT = 1, CARRY_TREE = 2 };
template <class Op, class T> struct carry_of { static constexpr int value = CARRY_SERIAL; };
template <bool COMP> struct carry_of<fold::op_sum<COMP>, float> { static constexpr int value = CARRY_EXACT; };
template <class T> struct carry_of<fold::op_val<0>, T> { static constexpr int value = CARRY_TREE; };
template <class T> struct carry_of<fold::op_val<1>, T> { static constexpr int value = CARRY_TREE; };
template <class T> struct carry_of<fold::op_val<3>, T> { static constexpr int value = CARRY_TREE; };
template <class T> struct carry_of<fold::op_val<4>, T> { static constexpr int value = CARRY_TREE; };

// Bytes of one published aggregate or prefix.
template <class Op, class T> constexpr size_t carry_bytes()
{
  return carry_of<Op, T>::value == CARRY_EXACT ? sizeof(xsum) : sizeof(state_of<Op, T>);
}

// Tiles of 64 KB, each split into 8 contiguous warp portions.  Pass 1: every
// warp folds its portion, the block folds the 8 portion totals into the tile's
// aggregate (and the portions' exclusive prefixes) and, when the column spans
// several tiles, publishes it; warp 0 then runs the look-back for the tile's
// prefix.  Pass 2: every warp rescans its own portion independently, in spans
// of 32 lanes x 8 consecutive 16-byte chunks moved through a padded
// shared-memory transpose (coalesced global accesses, no bank conflicts),
// re-reading the data from L2.  A block keeps two tiles in flight: it runs
// pass 1 of its next tile before the look-back of the current one, so the
// wait for the predecessors overlaps that read (two 64 KB tiles per block,
// about 80 MB in all, stay in the 129 MB L2).
template <class Op, class T>
struct scan_tiles {
  using S = state_of<Op, T>;
  static constexpr int CK = carry_of<Op, T>::value;
  static constexpr int CH = chunk_elems<T>();
  static constexpr int E = thread_elems<T>();
  static constexpr int SPAN = 32 * E;                      // elements per warp per span
  static constexpr int SPANS = 2;                          // spans per warp portion
  static constexpr int PORTION = SPAN * SPANS;             // elements per warp per tile
  static constexpr size_t TILE = (size_t)PORTION * kWarps; // elements per tile (64 KB)

  struct where {
    size_t k, tbase, tcnt;
    long long first;                                        // first tile of the column
  };
  __device__ __forceinline__ static where locate(const inner_shape& sh, unsigned long long t)
  {
    where w;
    const size_t j = (size_t)(t / sh.tiles_per_col);
    w.k = (size_t)(t % sh.tiles_per_col);
    const size_t r0 = w.k * TILE;
    w.tbase = j * sh.rows + r0;
    const size_t trem = sh.rows - r0;
    w.tcnt = trem < TILE ? trem : TILE;
    w.first = (long long)(t - w.k);
    return w;
  }

  // elements of warp `warp`'s portion that lie in the tile
  __device__ __forceinline__ static int portion_count(const where& w, int warp)
  {
    const long long c = (long long)w.tcnt - (long long)warp * PORTION;
    return c < 0 ? 0 : (c > PORTION ? PORTION : (int)c);
  }

  // Pass 1: the warps' portion totals, their exclusive prefixes (s_wex) and the
  // tile's aggregate (*out); thread 0 publishes the aggregate when `publish`.
  __device__ __forceinline__ static void aggregate(const T* x, const where& w, int vec, unsigned long long t,
                                                   bool publish, S* s_wtot, S* s_wex, S* out, xsum* xout,
                                                   unsigned* flags, S* agg, S* incl, xsum* xagg, xsum* xincl)
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int pc = portion_count(w, warp);
    const size_t pbase = w.tbase + (size_t)warp * PORTION;
    S c = Op::template init<T>();
    if (vec && pc == PORTION) {
      constexpr int L = PORTION / CH / 32;             // 16-byte loads per lane, 8 in flight
#pragma unroll 1
      for (int i0 = 0; i0 < L; i0 += 8) {
        uint4 g[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) g[i] = mem::ld_plain<16>(x + pbase + (size_t)((i0 + i) * 32 + lane) * CH).v;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const T* e = reinterpret_cast<const T*>(&g[i]);
#pragma unroll
          for (int q = 0; q < CH; ++q) Op::add(c, e[q]);
        }
      }
    } else {
      for (int e = lane; e < pc; e += 32) Op::add(c, x[pbase + (size_t)e]);
    }
    c = fold::warp_merge<Op, T>(c);
    if (lane == 0) s_wtot[warp] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      S a = Op::template init<T>();
      for (int ww = 0; ww < kWarps; ++ww) {
        s_wex[ww] = a;
        a = Op::merge(a, s_wtot[ww]);
      }
      *out = a;
      if (publish) publish_aggregate(a, w.k, t, flags, agg, incl, xagg, xincl, xout);
    }
    __syncthreads();
  }

  // Publish tile t's aggregate a: as its inclusive prefix when the tile starts
  // its column (k == 0), else as an aggregate.
  __device__ __forceinline__ static void publish_aggregate(const S& a, size_t k, unsigned long long t,
                                                           unsigned* flags, S* agg, S* incl, xsum* xagg,
                                                           xsum* xincl, xsum* xout)
  {
    const unsigned flag = k == 0 ? F_INCL : F_AGG;
    if constexpr (CK == CARRY_EXACT) {
      // the pair's value: s and c, or s alone once s is not finite (fold::result)
      xsum xa = xzero();
      xadd_float(xa, a.s);
      if (isfinite(a.s)) xadd_float(xa, a.c);
      xstore((k == 0 ? xincl : xagg) + t, xa);
      *xout = xa;   // the look-back adds it to the prefix it finds
    } else {
      (k == 0 ? incl : agg)[t] = a;
    }
    st_release(&flags[t], flag);
  }


  // Look-back (warp 0): the tile's prefix I(t-1) into *prefix and its inclusive
  // prefix published; false when a wait ran out or a predecessor failed.
  __device__ __forceinline__ static bool lookback(const where& w, unsigned long long t, const S& a, const xsum* xa, S* prefix,
                                                  unsigned* flags, S* agg, S* incl, xsum* xagg, xsum* xincl)
  {
    const int lane = threadIdx.x & 31;
    if (w.k == 0) {
      if (lane == 0) *prefix = Op::template init<T>();
      return true;
    }
    bool fail = false;
    if constexpr (CK == CARRY_EXACT) {
      // A round reads 32 * LB predecessors, LB per lane (tiles p0 - 32 j - lane):
      // their flags with relaxed loads issued together, one fence for the
      // acquire, then their values, so a round costs two round trips to L2
      // whatever LB is.
      constexpr int LB = 2;
      xsum ex = xzero();                             // exact sum of everything looked at so far
      long long p0 = (long long)t - 1;
      for (unsigned round = 0;; ++round) {
        unsigned f[LB];
#pragma unroll
        for (int j = 0; j < LB; ++j) {
          const long long p = p0 - 32 * j - lane;
          f[j] = p >= w.first ? ld_relaxed(&flags[p]) : F_INCL;   // before the column: an empty prefix
        }
        for (unsigned it = 0; it < kSpinMax; ++it) {
          bool pending = false;
#pragma unroll
          for (int j = 0; j < LB; ++j) pending |= f[j] == F_NONE;
          if (!pending) break;
          __nanosleep(64);
#pragma unroll
          for (int j = 0; j < LB; ++j)
            if (f[j] == F_NONE) f[j] = ld_relaxed(&flags[p0 - 32 * j - lane]);
        }
        fence_acquire();
        bool bad = false;
        unsigned incl_mask[LB];
#pragma unroll
        for (int j = 0; j < LB; ++j) {
          bad |= f[j] == F_NONE || f[j] == F_FAIL;
          incl_mask[j] = __ballot_sync(0xffffffffu, f[j] == F_INCL);
        }
        if (__any_sync(0xffffffffu, bad) || round >= kSpinMax) { fail = true; break; }
        int fl = 32 * LB;                            // nearest inclusive prefix in this window
#pragma unroll
        for (int j = LB - 1; j >= 0; --j)
          if (incl_mask[j]) fl = 32 * j + __ffs(incl_mask[j]) - 1;
        xsum v = xzero();
#pragma unroll
        for (int j = 0; j < LB; ++j) {
          const long long p = p0 - 32 * j - lane;
          if (p >= w.first && 32 * j + lane <= fl) xadd_into(v, (f[j] == F_AGG) ? xload(xagg + p) : xload(xincl + p));
        }
        xadd_into(ex, xwarp_sum(v));
        if (fl < 32 * LB) break;
        p0 -= 32 * LB;
      }
      if (!fail && lane == 0) {
        // publish first: successors wait on it, this tile's own prefix can follow
        xsum in = ex;
        xadd_into(in, *xa);
        xstore(xincl + t, in);
        st_release(&flags[t], F_INCL);
        *prefix = xto_pair(ex);
      }
    } else if constexpr (CK == CARRY_TREE) {
      // an exact operation: merge any window with a warp tree
      S ex = Op::template init<T>();
      long long p0 = (long long)t - 1;
      for (unsigned round = 0;; ++round) {
        const long long p = p0 - lane;
        unsigned f = F_INCL;
        S v = Op::template init<T>();
        if (p >= w.first) {
          f = wait_flag(&flags[p]);
          if (f == F_AGG) v = Op::ldcg(agg + p);
          else if (f == F_INCL) v = Op::ldcg(incl + p);
        }
        if (__any_sync(0xffffffffu, f == F_NONE || f == F_FAIL) || round >= kSpinMax) { fail = true; break; }
        const unsigned im = __ballot_sync(0xffffffffu, f == F_INCL);
        const int fl = im ? __ffs(im) - 1 : 32;
        if (lane > fl) v = Op::template init<T>();
        ex = Op::merge(fold::warp_merge<Op, T>(v), ex);
        if (fl < 32) break;
        p0 -= 32;
      }
      if (!fail && lane == 0) {
        *prefix = ex;
        incl[t] = Op::merge(ex, a);
        st_release(&flags[t], F_INCL);
      }
    } else {
      // Read the 32 nearest predecessors until one of them has published its
      // inclusive prefix; the prefix is then folded from at most 31 aggregates.
      const long long p = (long long)t - 1 - lane;
      int fl = 32;
      S val = Op::template init<T>();
      for (unsigned round = 0; fl == 32; ++round) {
        unsigned f = F_INCL;                         // before the column: the neutral prefix
        if (p >= w.first) {
          f = wait_flag(&flags[p]);
          if (f == F_AGG) val = Op::ldcg(agg + p);
          else if (f == F_INCL) val = Op::ldcg(incl + p);
        }
        if (__any_sync(0xffffffffu, f == F_NONE || f == F_FAIL) || round >= kSpinMax) { fail = true; break; }
        const unsigned im = __ballot_sync(0xffffffffu, f == F_INCL);
        fl = im ? __ffs(im) - 1 : 32;
        if (fl == 32) __nanosleep(128);
      }
      if (!fail) {
        // I(t-1) = fold of I(p) with A(p+1) ... A(t-1): lane fl holds I(p), lanes fl-1 .. 0 the aggregates
        S pre = Op::shfl_from(val, fl);
        for (int i = fl - 1; i >= 0; --i) pre = Op::merge(pre, Op::shfl_from(val, i));
        if (lane == 0) {
          *prefix = pre;
          incl[t] = Op::merge(pre, a);
          st_release(&flags[t], F_INCL);
        }
      }
    }
    if (fail && lane == 0) st_release(&flags[t], F_FAIL);
    return !fail;
  }



  // Pass 2: every warp rescans its portion from prefix (+) its portion prefix.
  __device__ __forceinline__ static void rescan(const T* x, T* y, const where& w, int vec, const S& prefix,
                                                const S& wex, bool failed, uint4* wb)
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* wbt = reinterpret_cast<T*>(wb);
    const int pc = portion_count(w, warp);
    S carry = Op::merge(prefix, wex);
    for (int sp = 0; sp < SPANS; ++sp) {
      const int s0 = sp * SPAN;
      if (s0 >= pc) break;
      const int cnt = (pc - s0) < SPAN ? pc - s0 : SPAN;
      const size_t base = w.tbase + (size_t)warp * PORTION + (size_t)s0;
      const bool full = vec && cnt == SPAN;
      if (full) {
        uint4 g[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) g[i] = mem::ld_stream<16>(x + base + (size_t)(i * 32 + lane) * CH).v;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int q = i * 32 + lane;
          wb[slot_of(q >> 3, q & 7)] = g[i];
        }
      } else {
        for (int e = lane; e < SPAN; e += 32) {
          const int q = e / CH;
          wbt[slot_of(q >> 3, q & 7) * CH + e % CH] = (e < cnt) ? x[base + (size_t)e] : T(0);
        }
      }
      __syncwarp();
      T v[E];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) *reinterpret_cast<uint4*>(&v[cc * CH]) = wb[slot_of(lane, cc)];
      const int mine = cnt - lane * E;
      S c = Op::template init<T>();
#pragma unroll
      for (int e = 0; e < E; ++e)
        if (full || e < mine) Op::add(c, v[e]);
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const S o = Op::shfl_from(c, lane >= d ? lane - d : 0);
        if (lane >= d) c = Op::merge(o, c);
      }
      S ex = Op::shfl_from(c, lane > 0 ? lane - 1 : 0);
      if (lane == 0) ex = Op::template init<T>();
      S st = Op::merge(carry, ex);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        Op::add(st, v[e]);
        v[e] = failed ? nan_value<T>() : (T)Op::finish(st, 0);
      }
      carry = Op::merge(carry, Op::shfl_from(c, 31));
      __syncwarp();
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) wb[slot_of(lane, cc)] = *reinterpret_cast<const uint4*>(&v[cc * CH]);
      __syncwarp();
      if (full) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int q = i * 32 + lane;
          mem::chunk<16> ch;
          ch.v = wb[slot_of(q >> 3, q & 7)];
          mem::st_stream<16>(y + base + (size_t)q * CH, ch);
        }
      } else {
        for (int e = lane; e < cnt; e += 32) {
          const int q = e / CH;
          y[base + (size_t)e] = wbt[slot_of(q >> 3, q & 7) * CH + e % CH];
        }
      }
      __syncwarp();
    }
  }
};

// Compensated FP32 sums (the exact-carry look-back) fit 64 registers without
// spilling: four blocks per SM then cover each other's look-back barriers.
template <class Op, class T> struct scan_min_blocks { static constexpr int value = 0; };
template <> struct scan_min_blocks<fold::op_sum<true>, float> { static constexpr int value = 4; };

template <class Op, class T>
__global__ void __launch_bounds__(256, (scan_min_blocks<Op, T>::value)) k_scan_inner(const T* __restrict__ x, T* __restrict__ y, inner_shape sh,
                                                    int vec, unsigned long long* __restrict__ ticket,
                                                    unsigned* __restrict__ flags, void* __restrict__ aggv,
                                                    void* __restrict__ inclv, unsigned* __restrict__ err)
{
  nt2cuda::mem::pdl_begin();
  using K = scan_tiles<Op, T>;
  using S = typename K::S;
  S* agg = reinterpret_cast<S*>(aggv);
  S* incl = reinterpret_cast<S*>(inclv);
  xsum* xagg = reinterpret_cast<xsum*>(aggv);
  xsum* xincl = reinterpret_cast<xsum*>(inclv);
  __shared__ __align__(16) uint4 s_buf[kWarps][32 * 9];
  __shared__ S s_wtot[kWarps];
  __shared__ S s_wex[2][kWarps];
  __shared__ S s_agg[2], s_prefix;
  __shared__ xsum s_xa[2];
  __shared__ unsigned long long s_tile[2];
  __shared__ int s_fail;
  const bool chained = sh.tiles_per_col > 1;
  const int warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) s_tile[0] = atomicAdd(ticket, 1ull);
  __syncthreads();
  unsigned long long t = s_tile[0];
  if (t >= sh.tiles) return;
  typename K::where w = K::locate(sh, t);
  K::aggregate(x, w, vec, t, chained, s_wtot, s_wex[0], &s_agg[0], &s_xa[0], flags, agg, incl, xagg, xincl);
  int slot = 0;
  for (;;) {
    // take the next tile and publish its aggregate before waiting on this one's predecessors
    if (threadIdx.x == 0) s_tile[slot ^ 1] = atomicAdd(ticket, 1ull);
    __syncthreads();
    const unsigned long long tn = s_tile[slot ^ 1];
    typename K::where wn{};
    if (tn < sh.tiles) {
      wn = K::locate(sh, tn);
      K::aggregate(x, wn, vec, tn, chained, s_wtot, s_wex[slot ^ 1], &s_agg[slot ^ 1], &s_xa[slot ^ 1], flags, agg,
                   incl, xagg, xincl);
    }
    if (threadIdx.x == 0) s_fail = 0;
    if (chained) {
      if (threadIdx.x < 32) {
        const bool ok = K::lookback(w, t, s_agg[slot], &s_xa[slot], &s_prefix, flags, agg, incl, xagg, xincl);
        if (!ok && threadIdx.x == 0) {
          s_fail = 1;
          atomicOr(err, 1u);
          atomicAdd(&g_wait_timeouts, 1ull);
        }
      }
    } else if (threadIdx.x == 0) {
      s_prefix = Op::template init<T>();
    }
    __syncthreads();
    K::rescan(x, y, w, vec, s_prefix, s_wex[slot][warp], s_fail != 0, s_buf[warp]);
    __syncthreads();   // s_prefix and s_fail are rewritten for the next tile
    if (tn >= sh.tiles) break;
    t = tn;
    w = wn;
    slot ^= 1;
  }
}

// Columns of at most one 32 KB tile (8 warps x 32 lanes x 8 consecutive
// 16-byte chunks): one pass, the tile read once into registers and scanned
// with no look-back.  (Chaining such register-held tiles through the
// look-back costs registers enough that the two-pass tiles above are faster
// for long columns on this GPU.)
template <class Op, class T>
__global__ void __launch_bounds__(256) k_scan_inner_1p(const T* __restrict__ x, T* __restrict__ y, inner_shape sh,
                                                       int vec, unsigned long long* __restrict__ ticket,
                                                       unsigned* __restrict__ flags, void* __restrict__ aggv,
                                                       void* __restrict__ inclv, unsigned* __restrict__ err)
{
  nt2cuda::mem::pdl_begin();
  using K = scan_tiles<Op, T>;
  using S = typename K::S;
  constexpr int CH = chunk_elems<T>();
  constexpr int E = thread_elems<T>();
  constexpr int SPAN = 32 * E;                      // elements per warp
  constexpr int TILE = kWarps * SPAN;
  __shared__ __align__(16) uint4 s_buf[kWarps][32 * 9];
  __shared__ S s_wex[kWarps];
  __shared__ S s_wtot[kWarps];
  __shared__ unsigned long long s_tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4* wb = s_buf[warp];
  T* wbt = reinterpret_cast<T*>(wb);

  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1ull);
    __syncthreads();
    const unsigned long long t = s_tile;
    if (t >= sh.tiles) break;
    typename K::where w;
    {
      const size_t j = (size_t)(t / sh.tiles_per_col);
      w.k = (size_t)(t % sh.tiles_per_col);
      const size_t r0 = w.k * (size_t)TILE;
      w.tbase = j * sh.rows + r0;
      const size_t trem = sh.rows - r0;
      w.tcnt = trem < (size_t)TILE ? trem : (size_t)TILE;
      w.first = (long long)(t - w.k);
    }
    const size_t base = w.tbase + (size_t)warp * SPAN;
    int cnt = (int)w.tcnt - warp * SPAN;
    cnt = cnt < 0 ? 0 : (cnt > SPAN ? SPAN : cnt);
    const bool full = vec && w.tcnt == (size_t)TILE;

    // ---- load the span (coalesced) into the lane-blocked layout, then registers
    if (full) {
      uint4 g[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) g[i] = mem::ld_stream<16>(x + base + (size_t)(i * 32 + lane) * CH).v;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int q = i * 32 + lane;
        wb[slot_of(q >> 3, q & 7)] = g[i];
      }
    } else {
      for (int e = lane; e < SPAN; e += 32) {
        const int q = e / CH;
        wbt[slot_of(q >> 3, q & 7) * CH + e % CH] = (e < cnt) ? x[base + (size_t)e] : T(0);
      }
    }
    __syncwarp();
    T v[E];
#pragma unroll
    for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(&v[c * CH]) = wb[slot_of(lane, c)];
    const int mine = cnt - lane * E;

    // ---- the thread's aggregate, the warp scan, the warp totals, the tile aggregate
    S c = Op::template init<T>();
#pragma unroll
    for (int e = 0; e < E; ++e)
      if (full || e < mine) Op::add(c, v[e]);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const S o = Op::shfl_from(c, lane >= d ? lane - d : 0);
      if (lane >= d) c = Op::merge(o, c);
    }
    if (lane == 31) s_wtot[warp] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      S a = Op::template init<T>();
      for (int ww = 0; ww < kWarps; ++ww) {
        s_wex[ww] = a;
        a = Op::merge(a, s_wtot[ww]);
      }
    }
    __syncthreads();

    // ---- outputs from the warp prefix and the lane prefix
    S ex = Op::shfl_from(c, lane > 0 ? lane - 1 : 0);
    if (lane == 0) ex = Op::template init<T>();
    S st = Op::merge(s_wex[warp], ex);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      Op::add(st, v[e]);
      v[e] = (T)Op::finish(st, 0);
    }
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) wb[slot_of(lane, cc)] = *reinterpret_cast<const uint4*>(&v[cc * CH]);
    __syncwarp();
    if (full) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int q = i * 32 + lane;
        mem::chunk<16> ch;
        ch.v = wb[slot_of(q >> 3, q & 7)];
        mem::st_stream<16>(y + base + (size_t)q * CH, ch);
      }
    } else {
      for (int e = lane; e < cnt; e += 32) {
        const int q = e / CH;
        y[base + (size_t)e] = wbt[slot_of(q >> 3, q & 7) * CH + e % CH];
      }
    }
    __syncthreads();   // shared state is rewritten by the next tile
  }
}

// Short columns (rows <= 64): one thread scans one column in index order.
template <class Op, class T>
__global__ void __launch_bounds__(256) k_scan_inner_short(const T* __restrict__ x, T* __restrict__ y, size_t rows,
                                                          size_t cols)
{
  nt2cuda::mem::pdl_begin();
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < cols; j += (size_t)gridDim.x * blockDim.x) {
    state_of<Op, T> st = Op::template init<T>();
    for (size_t r = 0; r < rows; ++r) {
      Op::add(st, x[j * rows + r]);
      y[j * rows + r] = (T)Op::finish(st, 0);
    }
  }
}

// ------------------------------------------------ TMA-staged row scans
// Row scans (dim 2) of tables with enough rows: each block owns a strip of
// 128 bytes of rows (32 floats or 16 doubles) and walks every column of it
// in order, so the table is read and written once and each row's running
// value stays on chip.  Thread 0 streams tiles of the strip (BR rows x 128
// columns, 16 KB) through STAGES shared-memory stages with
// cp.async.bulk.tensor; the threads split a tile's columns in NG groups of CG
// consecutive columns per row (thread t: row t % BR, group t / BR).  Per
// tile: every thread folds its CG values, the group totals of each row are
// folded in group order from the row's carry (group g stops after g of them:
// its prefix; the last group goes on to the next tile's carry, which it
// leaves in shared memory), every thread rescans its values from its prefix
// into the stage, and a TMA store writes the tile back.  Rows past the table
// and columns past its end read as zeros and are never stored (the tensor
// map clips both).  A stage is refilled once the store that last used it
// has read it.
template <class T> __host__ __device__ constexpr int outer_tma_rows() { return 128 / (int)sizeof(T); }
constexpr int kOuterTmaCols = 128;

struct outer_tma_shape {
  size_t rows, cols, strips, ctiles;
  uint32_t wait_rounds;
};

template <class Op, class T, int STAGES>
__global__ void __launch_bounds__(256) k_scan_outer_tma(const __grid_constant__ CUtensorMap xmap,
                                                        const __grid_constant__ CUtensorMap ymap, outer_tma_shape sh)
{
  nt2cuda::mem::pdl_begin();
  using S = state_of<Op, T>;
  constexpr int BR = outer_tma_rows<T>(), BC = kOuterTmaCols;
  constexpr int NG = 256 / BR, CG = BC / NG;
  constexpr uint32_t TBYTES = (uint32_t)(BR * BC * sizeof(T));
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* stage0 = reinterpret_cast<T*>(smem_raw);          // [STAGES][BC][BR], column-major boxes
  __shared__ __align__(8) uint64_t full[STAGES];
  __shared__ S s_tot[NG][BR];
  __shared__ S s_carry[2][BR];
  const int r = threadIdx.x % BR, g = threadIdx.x / BR;
  const int row0 = (int)(blockIdx.x * BR);

  if (threadIdx.x == 0) {
    for (int st = 0; st < STAGES; ++st) tma::mbar_init(&full[st], 1);
    tma::fence_barrier_init();
    for (int st = 0; st < STAGES - 1 && (size_t)st < sh.ctiles; ++st) {
      tma::mbar_arrive_expect_tx(&full[st], TBYTES);
      tma::tensor_g2s_2d(stage0 + (size_t)st * BR * BC, &xmap, row0, st * BC, &full[st]);
    }
  }
  __syncthreads();

  if (threadIdx.x < BR) s_carry[0][threadIdx.x] = Op::template init<T>();
  for (size_t k = 0; k < sh.ctiles; ++k) {
    const int st = (int)(k % STAGES);
    T* buf = stage0 + (size_t)st * BR * BC;
    const bool ok = tma::mbar_wait(&full[st], (uint32_t)((k / STAGES) & 1u), sh.wait_rounds);
    if (__syncthreads_or(!ok)) {
      // a copy that never landed: wait (bounded) for the rest, leave the
      // strip's outputs from here on unwritten and count the failure
      if (threadIdx.x == 0) {
        atomicAdd(&g_wait_timeouts, 1ull);
        for (size_t q = k + 1; q < k + STAGES - 1 && q < sh.ctiles; ++q)
          tma::mbar_wait(&full[q % STAGES], (uint32_t)((q / STAGES) & 1u), sh.wait_rounds);
        tma::bulk_wait<0>();
      }
      return;
    }
    T v[CG];
#pragma unroll
    for (int i = 0; i < CG; ++i) v[i] = buf[(g * CG + i) * BR + r];
    S tot = Op::template init<T>();
#pragma unroll
    for (int i = 0; i < CG; ++i) Op::add(tot, v[i]);
    s_tot[g][r] = tot;
    __syncthreads();
    // this group's prefix (and, in the last group, the next tile's carry),
    // folded in group order; g is the same across a warp
    S pre = s_carry[k & 1][r];
    for (int gg = 0; gg < g; ++gg) pre = Op::merge(pre, s_tot[gg][r]);
    if (g == NG - 1) s_carry[(k + 1) & 1][r] = Op::merge(pre, s_tot[g][r]);
#pragma unroll
    for (int i = 0; i < CG; ++i) {
      Op::add(pre, v[i]);
      v[i] = (T)Op::finish(pre, 0);
    }
#pragma unroll
    for (int i = 0; i < CG; ++i) buf[(g * CG + i) * BR + r] = v[i];
    tma::fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma::tensor_s2g_2d(&ymap, row0, (int)(k * BC), buf);
      tma::bulk_commit();
      // refill the stage of the previous tile once its store has read it
      const size_t nk = k + STAGES - 1;
      if (nk < sh.ctiles) {
        tma::bulk_wait_read<1>();
        const int ns = (int)(nk % STAGES);
        tma::mbar_arrive_expect_tx(&full[ns], TBYTES);
        tma::tensor_g2s_2d(stage0 + (size_t)ns * BR * BC, &xmap, row0, (int)(nk * BC), &full[ns]);
      }
    }
  }
  if (threadIdx.x == 0) tma::bulk_wait<0>();
}

// ------------------------------------------------------------ outer scan
// A block owns a strip of 32*V rows per warp (8 warps: 256*V rows) and a chunk
// of columns; each thread walks its V rows through the chunk's columns in
// order.  Pass 1 (WRITE = false) stores each row's chunk total; pass 2
// starts each row from the left fold of the earlier chunks' totals and writes
// the running values.
struct outer_shape {
  size_t rows, cols, cchunk, chunks, strips;
};

template <class Op, class T, int V, bool WRITE>
__global__ void __launch_bounds__(256) k_scan_outer(const T* __restrict__ x, T* __restrict__ y, outer_shape sh,
                                                    state_of<Op, T>* __restrict__ totals)
{
  nt2cuda::mem::pdl_begin();
  using S = state_of<Op, T>;
  constexpr int ROWS = 256 * V;
  const size_t units = sh.strips * sh.chunks;
  for (size_t u = blockIdx.x; u < units; u += gridDim.x) {
    const size_t strip = u / sh.chunks, c = u % sh.chunks;
    const size_t row0 = strip * ROWS + (size_t)threadIdx.x * V;
    if (row0 >= sh.rows) continue;
    const size_t m0 = c * sh.cchunk;
    const size_t m1 = (m0 + sh.cchunk < sh.cols) ? m0 + sh.cchunk : sh.cols;
    const bool vrow = row0 + V <= sh.rows;
    S st[V];
#pragma unroll
    for (int l = 0; l < V; ++l) st[l] = Op::template init<T>();
    if constexpr (WRITE) {
      // prefix of this chunk: the left fold of the earlier chunks' totals (k_scan_outer_prefix)
      if (totals)
#pragma unroll
        for (int l = 0; l < V; ++l)
          if (row0 + l < sh.rows) st[l] = Op::ldcg(totals + (strip * sh.chunks + c) * ROWS + threadIdx.x * V + l);
    }
    size_t m = m0;
    if (vrow) {
      constexpr int U = 8;
      for (; m + U <= m1; m += U) {
        T v[U][V];
#pragma unroll
        for (int uu = 0; uu < U; ++uu) mem::load_vec<T, V, true>(x, (m + uu) * sh.rows + row0, v[uu]);
#pragma unroll
        for (int uu = 0; uu < U; ++uu) {
          T o[V];
#pragma unroll
          for (int l = 0; l < V; ++l) {
            Op::add(st[l], v[uu][l]);
            o[l] = (T)Op::finish(st[l], 0);
          }
          if constexpr (WRITE) mem::store_vec<T, V>(y, (m + uu) * sh.rows + row0, o);
        }
      }
    }
    for (; m < m1; ++m)
#pragma unroll
      for (int l = 0; l < V; ++l)
        if (row0 + l < sh.rows) {
          Op::add(st[l], x[m * sh.rows + row0 + l]);
          if constexpr (WRITE) y[m * sh.rows + row0 + l] = (T)Op::finish(st[l], 0);
        }
    if constexpr (!WRITE) {
#pragma unroll
      for (int l = 0; l < V; ++l)
        if (row0 + l < sh.rows) totals[(strip * sh.chunks + c) * ROWS + threadIdx.x * V + l] = st[l];
    }
  }
}

// Between the passes: replace each row's chunk totals by their exclusive left
// folds, in chunk order (one thread per row of a strip).
template <class Op, class T, int V>
__global__ void __launch_bounds__(256) k_scan_outer_prefix(outer_shape sh, state_of<Op, T>* __restrict__ totals)
{
  nt2cuda::mem::pdl_begin();
  using S = state_of<Op, T>;
  constexpr size_t ROWS = 256 * (size_t)V;
  const size_t n = sh.strips * ROWS;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t strip = i / ROWS, r = i % ROWS;
    S run = Op::template init<T>();
    for (size_t c = 0; c < sh.chunks; ++c) {
      S* p = totals + (strip * sh.chunks + c) * ROWS + r;
      const S t = *p;
      *p = run;
      run = Op::merge(run, t);
    }
  }
}

}  // namespace scan
}  // namespace nt2cuda
