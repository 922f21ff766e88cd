// nt2cuda/bs_x2.cuh -- NT2's float exp, log, erfc, normcdf, pow and cbrt,
// two lanes at a time on Blackwell's packed FP32 instructions, bit-identical to
// the one-lane forms of math.cuh.
//
// sm_100-family SMs execute add.rn.f32x2 / mul.rn.f32x2 on a 64-bit
// register pair at the issue cost of one scalar FP32 instruction, each half
// rounded exactly as the scalar add or multiply.  NT2's exact arithmetic is
// nothing but correctly rounded adds, multiplies, divisions and square roots
// (its fma/fnms are a*b+c rounded twice), so the same sequence run on
// register pairs gives, lane by lane, the same bits for half the issue
// slots.  What does not pack stays per lane: comparisons, selects,
// exponent-bit arithmetic and the special-function unit.  The functors take
// F as math.cuh's do: F = true makes each NT2 fma/fnms (and Horner step) one
// fma.rn.f32x2, the fused precision mode's arithmetic.
//
// Beyond packing, the steps below are rearranged only where the result is
// provably the same:
//  * rint(v) for |v| <= 2^22 is (v + 1.5*2^23) - 1.5*2^23, and the sum's low
//    bits are the integer itself, so exp needs neither the FP32-to-integer
//    conversion nor the round instruction (both on the slow XU pipe); lanes
//    outside that range are the ones exp's selections replace.
//  * exp's `a0 != a0 ? a0 : r` is dropped: a NaN argument already makes the
//    computed r NaN (NaN payloads are not part of the results' contract; the
//    CPU and the GPU make different ones).
//  * z = x/(1+x) inside erfc uses one reciprocal approximation, a Newton step
//    and Markstein's correction of the quotient (P. Markstein, "IA-64 and
//    Elementary Functions", 2000: with y within half an ulp of 1/b and q
//    within an ulp of a/b, q + (a - b q) y rounds to a/b); x is first clamped
//    to 2^64, where x/(1+x) is already exactly 1, which keeps every step
//    normal.  The quotient, and erfc as a whole, are checked bit for bit
//    against the one-lane form over every non-negative float.
//  * log takes a branch-free path when every lane of the warp has a positive,
//    normal, finite argument (no denormal rescale, no special values) and the
//    one-lane form otherwise.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "math.cuh"

namespace nt2cuda {
namespace x2 {

using math::fbits;
using math::cf;

// add, sub, mul and fma are spelled in PTX with an explicit rounding
// modifier.  Unlike the scalar forms, that does not keep ptxas from merging
// a packed multiply whose only use is a packed add or subtract into one
// fused operation, which rounds once and changes NT2's twice-rounded result
// (seen on sm_103a with CUDA 13.0; -fmad=false does not stop it).  So every
// product that is an operand of an add or a subtract is formed by mul_r:
// fma(a, b, z) with z = -0 read from constant memory, which is a*b rounded
// once (a*b + (-0) is a*b, the sign of a zero product included) and which
// the code generator cannot merge with the add, since it does not know z.
// Plain mul is kept for products that feed only multiplies, divisions,
// comparisons and selections.
__constant__ float c_x2_negzero = -0.0f;

__device__ __forceinline__ float2 splat(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add(float2 a, float2 b)
{
  float2 r;
  asm("{.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
      "add.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 sub(float2 a, float2 b)
{
  float2 r;
  asm("{.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
      "sub.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 mul(float2 a, float2 b)
{
  float2 r;
  asm("{.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
      "mul.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c)
{
  float2 r;
  asm("{.reg .b64 a, b, c, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tmov.b64 c, {%6, %7};\n\t"
      "fma.rn.f32x2 d, a, b, c;\n\tmov.b64 {%0, %1}, d;}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}
// a*b rounded once, as an operand of a later add or subtract (see above)
__device__ __forceinline__ float2 mul_r(float2 a, float2 b) { return fma(a, b, splat(c_x2_negzero)); }
// NT2's fma / fnms: a*b+c and c-a*b, each rounded twice (F = false), or
// one hardware FMA each (F = true, math::madd<true> / nmsub<true>)
template <bool F> __device__ __forceinline__ float2 madd(float2 a, float2 b, float2 c)
{
  if constexpr (F) return fma(a, b, c);
  else return add(mul_r(a, b), c);
}
template <bool F> __device__ __forceinline__ float2 nmsub(float2 a, float2 b, float2 c)
{
  if constexpr (F) return fma(make_float2(-a.x, -a.y), b, c);
  else return sub(c, mul_r(a, b));
}

template <bool F, int N>
__device__ __forceinline__ float2 horner(float2 x, const uint32_t (&c)[N])
{
  float2 acc = splat(fbits(c[0]));
#pragma unroll
  for (int i = 1; i < N; ++i) acc = madd<F>(x, acc, splat(fbits(c[i])));
  return acc;
}

constexpr float kRound = 12582912.0f;   // 1.5 * 2^23

// 2^k as a float from t = k + 1.5*2^23 (|k| <= 127): the low bits of t's
// pattern are k, and (k + 127) << 23 is the pattern of 2^k.
__device__ __forceinline__ float scale_from_rounded(float t)
{
  return __uint_as_float((__float_as_uint(t) << 23) + 0x3f800000u);
}

// exp's reduction and polynomial (math::exp) before its selections:
// returns c * 2^k with k = rint(a0 / ln 2); exact for minlog < a0 < maxlog.
template <bool F> __device__ __forceinline__ float2 exp_core(float2 a0)
{
  constexpr uint32_t P[5] = {0x3ab778cfu, 0x3c098d8bu, 0x3d2aa957u, 0x3e2aa9a5u, 0x3f000000u};
  const float2 t = add(mul_r(splat(fbits(cf::invlog_2)), a0), splat(kRound));
  const float2 k = sub(t, splat(kRound));
  float2 x = nmsub<F>(k, splat(fbits(cf::log_2hi)), a0);
  x = nmsub<F>(k, splat(fbits(cf::log_2lo)), x);
  const float2 y = horner<F>(x, P);
  const float2 c = add(madd<F>(y, mul(x, x), x), splat(1.0f));
  return mul(c, make_float2(scale_from_rounded(t.x), scale_from_rounded(t.y)));
}

// NT2's float exp (math::exp), two lanes.
template <bool F> __device__ __forceinline__ float2 exp(float2 a0)
{
  float2 r = exp_core<F>(a0);
  const float lo = fbits(cf::minlog), hi = fbits(cf::maxlog), inf = __int_as_float(0x7f800000);
  r.x = (a0.x <= lo) ? 0.0f : r.x;
  r.y = (a0.y <= lo) ? 0.0f : r.y;
  r.x = (a0.x >= hi) ? inf : r.x;
  r.y = (a0.y >= hi) ? inf : r.y;
  return r;
}

// NT2's float log (math::log), two lanes.
__device__ __forceinline__ bool log_fast_ok(float a)
{
  return __float_as_uint(a) - 0x00800000u < 0x7f000000u;   // positive, normal, finite
}
template <bool F> __device__ __forceinline__ float2 log(float2 a0)
{
  if (!__all_sync(__activemask(), log_fast_ok(a0.x) && log_fast_ok(a0.y)))
    return make_float2(math::log<F>(a0.x), math::log<F>(a0.y));
  constexpr uint32_t P[8] = {0xbda5dff0u, 0x3e0229f9u, 0xbe04d6b7u, 0x3e116e80u,
                             0xbe2a6aa0u, 0x3e4cd0a3u, 0xbe800064u, 0x3eaaaaa9u};
  const uint32_t u0 = __float_as_uint(a0.x), u1 = __float_as_uint(a0.y);
  float2 x = make_float2(__uint_as_float((u0 & 0x007fffffu) | 0x3f000000u),
                         __uint_as_float((u1 & 0x007fffffu) | 0x3f000000u));   // fast_frexp mantissa
  const bool lt0 = x.x < fbits(cf::sqrt_2o_2), lt1 = x.y < fbits(cf::sqrt_2o_2);
  // fe = e, or e - 1 below sqrt(2)/2, e = biased exponent - 126, as a float:
  // (e + 1.5*2^23) - 1.5*2^23, the integer placed in the sum's low bits
  const float2 fe = sub(make_float2(__uint_as_float((u0 >> 23) + (0x4b400000u - 126u) - (lt0 ? 1u : 0u)),
                                    __uint_as_float((u1 >> 23) + (0x4b400000u - 126u) - (lt1 ? 1u : 0u))),
                        splat(kRound));
  x = sub(mul_r(x, make_float2(lt0 ? 2.0f : 1.0f, lt1 ? 2.0f : 1.0f)), splat(1.0f));
  const float2 x2 = mul(x, x);
  float2 y = mul_r(mul(horner<F>(x, P), x), x2);
  y = madd<F>(fe, splat(fbits(cf::log_2lo)), y);
  y = madd<F>(splat(-0.5f), x2, y);
  return madd<F>(splat(fbits(cf::log_2hi)), fe, add(add(x, y), splat(0.0f)));
}

// x/(1+x) for x >= 0 (and NaN), as __fdiv_rn(x, 1+x) with x clamped to 2^64
// (see the header comment); the reciprocals are per lane.
// a/b for normal b and a quotient that stays normal (or is zero): one
// reciprocal approximation per lane, a Newton step for 1/b, then Markstein's
// correction of q = a*(1/b) (see the header comment).  Where it is used, its
// agreement with the IEEE division is checked over every input it can get.
__device__ __forceinline__ float2 markstein_quot(float2 a, float2 b)
{
  float2 y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y.x) : "f"(b.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y.y) : "f"(b.y));
  const float2 nb = make_float2(-b.x, -b.y);
  const float2 e = fma(nb, y, splat(1.0f));
  y = fma(y, e, y);
  const float2 q = mul(a, y);
  const float2 r = fma(nb, q, a);
  return fma(r, y, q);
}

__device__ __forceinline__ float2 x_over_1px(float2 x)
{
  const float2 a = make_float2(fminf(x.x, 18446744073709551616.0f), fminf(x.y, 18446744073709551616.0f));
  return markstein_quot(a, add(splat(1.0f), a));
}

// The two regions of NT2's float erfc (math::erfc_small / erfc_large) on
// z = x/(1+x), and the final selection for x = inf.
template <bool F> __device__ __forceinline__ float2 erfc_small(float2 z)
{
  constexpr uint32_t P3[9] = {0x41aa8e55u, 0x401b5680u, 0xc010d956u, 0x3f2cff3bu,
                              0xc016c985u, 0xbffc9284u, 0xbfa11698u, 0xbe036d7eu, 0x3f7ffffeu};
  return mul(sub(splat(1.0f), z), horner<F>(z, P3));
}
template <bool F> __device__ __forceinline__ float2 erfc_large(float2 x, float2 z)
{
  constexpr uint32_t P2[11] = {0xc0283611u, 0x40d67e3bu, 0xc0cd1a85u, 0x4050b063u,
                               0xbfaea865u, 0x3e2006f0u, 0x3e1175c7u, 0x3ec4ca6eu,
                               0x3e243828u, 0xbf918a62u, 0x3f0a0e8bu};
  // exp(-x*x): the argument is <= 0, so only the underflow selection applies
  const float2 m = mul_r(x, x);
  const float2 na = make_float2(-m.x, -m.y);
  float2 ex = exp_core<F>(na);
  const float lo = fbits(cf::minlog);
  ex.x = (na.x <= lo) ? 0.0f : ex.x;
  ex.y = (na.y <= lo) ? 0.0f : ex.y;
  return mul(ex, horner<F>(sub(z, splat(0.4f)), P2));
}
__device__ __forceinline__ float2 erfc_finish(float2 x, float2 r)
{
  const float inf = __int_as_float(0x7f800000);
  r.x = (x.x == inf) ? 0.0f : r.x;
  r.y = (x.y == inf) ? 0.0f : r.y;
  return r;
}

// NT2's float erfc of x = |a| (math::erfc_abs), two lanes, both regions
// computed and the right one selected per lane.
template <bool F> __device__ __forceinline__ float2 erfc_abs(float2 x)
{
  const float2 z = x_over_1px(x);
  const float2 small = erfc_small<F>(z), large = erfc_large<F>(x, z);
  const float two3 = fbits(cf::twothird);
  return erfc_finish(x, make_float2((x.x < two3) ? small.x : large.x, (x.y < two3) ? small.y : large.y));
}

// The same for a pair whose lanes are known to lie in one region (region 0:
// both x < 2/3, 1: both not), or not (2): only the regions needed run, and
// each lane gets what erfc_abs gives it.
template <bool F> __device__ __forceinline__ float2 erfc_abs_region(float2 x, int region)
{
  const float2 z = x_over_1px(x);
  if (region == 0) return erfc_finish(x, erfc_small<F>(z));
  if (region == 1) return erfc_finish(x, erfc_large<F>(x, z));
  return erfc_abs<F>(x);
}

// normcdf(a) and normcdf(-a) from erfc of |y|, y = -a sqrt(2)/2 (math::normcdf_pair).
__device__ __forceinline__ float2 normcdf_arg(float2 a0) { return mul(splat(-fbits(cf::sqrt_2o_2)), a0); }
__device__ __forceinline__ void normcdf_from_erfc(float2 y, float2 r1, float2& pos, float2& neg)
{
  const float2 two_m = sub(splat(2.0f), r1);
  pos = mul(splat(0.5f), make_float2((y.x < 0.0f) ? two_m.x : r1.x, (y.y < 0.0f) ? two_m.y : r1.y));
  neg = mul(splat(0.5f), make_float2((y.x > 0.0f) ? two_m.x : r1.x, (y.y > 0.0f) ? two_m.y : r1.y));
}
template <bool F> __device__ __forceinline__ void normcdf_pair(float2 a0, float2& pos, float2& neg)
{
  const float2 y = normcdf_arg(a0);
  normcdf_from_erfc(y, erfc_abs<F>(make_float2(fabsf(y.x), fabsf(y.y))), pos, neg);
}

// The Black-Scholes statement of nt2cuda/blackscholes.cuh (exact mode,
// normcdf via erfc) for two options, c = fma(sqr(v), 0.5, r), in two halves
// around the erfc evaluations: bs_front gives the normcdf arguments y1, y2
// (of d1 and d2) and e = K exp(-r T); bs_back the prices from erfc(|y1|),
// erfc(|y2|).
template <bool F>
__device__ __forceinline__ void bs_d(float2 S, float2 K, float2 T, float r, float v, float c, float2& d1, float2& d2,
                                     float2& e)
{
  const float2 da = make_float2(__fsqrt_rn(T.x), __fsqrt_rn(T.y));
  const float2 vda = mul_r(splat(v), da);
  const float2 q = make_float2(__fdiv_rn(S.x, K.x), __fdiv_rn(S.y, K.y));
  const float2 num = madd<F>(splat(c), T, log<F>(q));
  d1 = make_float2(__fdiv_rn(num.x, vda.x), __fdiv_rn(num.y, vda.y));
  d2 = sub(d1, vda);
  e = mul(K, exp<F>(mul_r(splat(-r), T)));
}
template <bool F>
__device__ __forceinline__ void bs_front(float2 S, float2 K, float2 T, float r, float v, float c, float2& y1,
                                         float2& y2, float2& e)
{
  float2 d1, d2;
  bs_d<F>(S, K, T, r, v, c, d1, d2, e);
  y1 = normcdf_arg(d1);
  y2 = normcdf_arg(d2);
}
template <bool F>
__device__ __forceinline__ void bs_back(float2 S, float2 e, float2 y1, float2 r1, float2 y2, float2 r2, float2& call,
                                        float2& put)
{
  float2 n1, m1, n2, m2;
  normcdf_from_erfc(y1, r1, n1, m1);
  normcdf_from_erfc(y2, r2, n2, m2);
  call = nmsub<F>(e, n2, mul_r(S, n1));
  put = nmsub<F>(S, m1, mul_r(e, m2));
}
template <bool F>
__device__ __forceinline__ void blackscholes(float2 S, float2 K, float2 T, float r, float v, float c, float2& call,
                                             float2& put)
{
  float2 y1, y2, e;
  bs_front<F>(S, K, T, r, v, c, y1, y2, e);
  bs_back<F>(S, e, y1, erfc_abs<F>(make_float2(fabsf(y1.x), fabsf(y1.y))), y2,
             erfc_abs<F>(make_float2(fabsf(y2.x), fabsf(y2.y))), call, put);
}

// ------------------------------------------------------------ fast mode
// The fast precision mode's functors (math::fast) two lanes at a time: the
// special-function-unit steps (ex2, lg2, rsqrt, the reciprocal divisions) per
// lane, every FMA, multiply and add packed; a product that feeds an add is
// formed by mul_r as above, so each lane gets the one-lane function's bits.
namespace fast {

__device__ __forceinline__ float2 ex2(float2 x) { return make_float2(math::fast::ex2(x.x), math::fast::ex2(x.y)); }

__device__ __forceinline__ float2 exp_small(float2 x) { return ex2(mul(x, splat(1.4426950408889634f))); }

__device__ __forceinline__ float2 log(float2 a0)
{
  const float2 r0 = mul(make_float2(math::fast::lg2(a0.x), math::fast::lg2(a0.y)), splat(0.69314718055994530942f));
  float r[2] = {r0.x, r0.y};
  const float a[2] = {a0.x, a0.y};
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    r[l] = (a[l] < 0.0f || a[l] != a[l]) ? __int_as_float(0x7fffffff) : r[l];
    r[l] = (a[l] == __int_as_float(0x7f800000)) ? a[l] : r[l];
    r[l] = (a[l] == 0.0f) ? __int_as_float(0xff800000) : r[l];
  }
  return make_float2(r[0], r[1]);
}

__device__ __forceinline__ float2 erfc_abs_nr(float2 x)
{
  const float2 y = fma(splat(0.5f), x, splat(1.0f));
  const float2 t = make_float2(__fdividef(1.0f, y.x), __fdividef(1.0f, y.y));
  float2 p = splat(0.17087277f);
  p = fma(p, t, splat(-0.82215223f));
  p = fma(p, t, splat(1.48851587f));
  p = fma(p, t, splat(-1.13520398f));
  p = fma(p, t, splat(0.27886807f));
  p = fma(p, t, splat(-0.18628806f));
  p = fma(p, t, splat(0.09678418f));
  p = fma(p, t, splat(0.37409196f));
  p = fma(p, t, splat(1.00002368f));
  p = fma(p, t, splat(-1.26551223f));
  return mul_r(t, exp_small(fma(make_float2(-x.x, -x.y), x, p)));
}

__device__ __forceinline__ void normcdf_pair(float2 a0, float2& pos, float2& neg)
{
  const float2 y = mul(splat(-fbits(cf::sqrt_2o_2)), a0);
  const float2 r1 = erfc_abs_nr(make_float2(fabsf(y.x), fabsf(y.y)));
  const float2 two_m = sub(splat(2.0f), r1);
  pos = mul(splat(0.5f), make_float2((y.x < 0.0f) ? two_m.x : r1.x, (y.y < 0.0f) ? two_m.y : r1.y));
  neg = mul(splat(0.5f), make_float2((-y.x < 0.0f) ? two_m.x : r1.x, (-y.y < 0.0f) ? two_m.y : r1.y));
}

// bs_lane's fast branch (normcdf), two options
__device__ __forceinline__ void blackscholes(float2 S, float2 K, float2 T, float r, float v, float c, float2& call,
                                             float2& put)
{
  const float2 rs = make_float2(rsqrtf(T.x), rsqrtf(T.y));
  const float2 vda = mul_r(splat(v), mul(T, rs));
  const float2 q = log(make_float2(__fdividef(S.x, K.x), __fdividef(S.y, K.y)));
  const float2 num = fma(splat(c), T, q);
  const float2 d1 = make_float2(__fdividef(num.x, vda.x), __fdividef(num.y, vda.y));
  const float2 d2 = sub(d1, vda);
  const float2 e = mul(K, exp_small(mul(splat(-r), T)));
  float2 n1, m1, n2, m2;
  normcdf_pair(d1, n1, m1);
  normcdf_pair(d2, n2, m2);
  call = fma(make_float2(-e.x, -e.y), n2, mul(S, n1));
  put = fma(make_float2(-S.x, -S.y), m1, mul(e, m2));
}

}  // namespace fast

// NT2's fastnormcdf(a) and fastnormcdf(-a) (math::fastnormcdf_pair), two
// lanes; the reciprocal is the IEEE division per lane.
template <bool F> __device__ __forceinline__ void fastnormcdf_pair(float2 a0, float2& pos, float2& neg)
{
  constexpr uint32_t P[5] = {0x3faa466fu, 0xbfe91eeau, 0x3fe40778u, 0xbeb68f87u, 0x3ea385fau};
  const float2 l = make_float2(fabsf(a0.x), fabsf(a0.y));
  const float2 den = madd<F>(splat(0.2316419f), l, splat(1.0f));
  const float2 k = make_float2(__fdiv_rn(1.0f, den.x), __fdiv_rn(1.0f, den.y));
  const float2 ll = mul(l, l);
  const float2 w = mul_r(horner<F>(k, P),
                         mul(mul(k, splat(fbits(cf::invsqrt_2pi))), exp<F>(mul(make_float2(-ll.x, -ll.y), splat(0.5f)))));
  const float2 om = sub(splat(1.0f), w);
  pos = make_float2((a0.x > 0.0f) ? om.x : w.x, (a0.y > 0.0f) ? om.y : w.y);
  neg = make_float2((-a0.x > 0.0f) ? om.x : w.x, (-a0.y > 0.0f) ? om.y : w.y);
}

// The statement with fastnormcdf (the demo form's cdf), two options.
template <bool F>
__device__ __forceinline__ void blackscholes_fastnormcdf(float2 S, float2 K, float2 T, float r, float v, float c,
                                                         float2& call, float2& put)
{
  float2 d1, d2, e, n1, m1, n2, m2;
  bs_d<F>(S, K, T, r, v, c, d1, d2, e);
  fastnormcdf_pair<F>(d1, n1, m1);
  fastnormcdf_pair<F>(d2, n2, m2);
  call = nmsub<F>(e, n2, mul_r(S, n1));
  put = nmsub<F>(S, m1, mul_r(e, m2));
}

// ------------------------------------------------------------------- pow
// NT2's float pow and pow_abs (math::pow, math::pow_abs), two lanes.  Per
// lane: frexp, the table index and the table reads, the integer-to-float
// conversions, the floors, the float-to-integer step, the exponent bits of
// ldexp and the special cases.  Packed: every add, subtract, multiply and
// NT2 fma.  The one division, of the reduced mantissa by its table value
// A[i] in [1/2, 1], is markstein_quot; its operands depend on the mantissa
// of a0 alone, so a check over every float a0 covers every quotient that
// pow forms.  A warp whose lanes all have ordinary arguments (a0 positive,
// or any sign for pow_abs, normal and finite; a1 finite) skips the zero,
// infinity and sign selections, which cannot apply to them.
__device__ __forceinline__ float2 pow_reduc(float2 x)
{
  // 1/16 * floor(16 x): both products are exact (powers of two, no overflow
  // where the result is kept), so how they are scheduled cannot change them
  const float2 t = mul(splat(16.0f), x);
  return mul(splat(0.0625f), make_float2(floorf(t.x), floorf(t.y)));
}

// Boost.SIMD ldexp as math::pow_ldexp, the two multiplies packed
__device__ __forceinline__ float2 pow_ldexp(float2 a, int e0, int e1)
{
  using C = math::powc<float>;
  float s[2], f[2];
  const int ein[2] = {e0, e1};
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    int e = ein[l];
    const bool den = e < C::mine;
    e = den ? e - C::mine : e;
    float fl = den ? C::bits(C::smallest) : 1.0f;
    const bool test = e == C::lime;
    fl = test ? math::add(fl, 1.0f) : fl;
    e = test ? e - 1 : e;
    s[l] = C::bits((C::U)(unsigned)(e + C::maxe) << C::nbm);
    f[l] = fl;
  }
  return mul(mul(a, make_float2(s[0], s[1])), make_float2(f[0], f[1]));
}

// math::pow_abs's selections after the arithmetic, one lane
__device__ __forceinline__ float pow_special(float a0, float a1, float z, bool zer_ret, bool inf_ret)
{
  const float ax = fabsf(a0);
  const bool gtax1 = ax > 1.0f;
  const float inf = __int_as_float(0x7f800000);
  if (a1 == inf) z = gtax1 ? inf : 0.0f;
  if (a1 == -inf) z = gtax1 ? 0.0f : inf;
  if (ax == inf) z = a1 > 0.0f ? inf : (a1 < 0.0f ? 0.0f : 1.0f);
  if (zer_ret) z = 0.0f;
  if (inf_ret) z = inf;
  if (ax == 1.0f) z = ax;
  return a0 == 0.0f ? (a1 == 0.0f ? 1.0f : 0.0f) : z;
}

// PLAIN: every lane's |a0| is normal and finite and its a1 finite, where
// frexp is the bit split alone and the only selections that can apply are
// the range results and |a0| = 1 (the others test for zeros and infinities).
template <bool F, bool PLAIN> __device__ __forceinline__ float2 pow_abs_core(float2 a0, float2 a1)
{
  using C = math::powc<float>;
  constexpr uint32_t P1[4] = {0xbe2a61b2u, 0x3e4d2fa3u, 0xbe800015u, 0x3eaaaaa3u};   // math::pow1
  constexpr uint32_t P2[4] = {0x3c1a49bcu, 0x3d634d38u, 0x3e75fde1u, 0x3f317218u};   // math::pow2
  int e[2], i[2];
  float2 x;
  if constexpr (PLAIN) {
    const uint32_t b0 = __float_as_uint(a0.x) & 0x7fffffffu, b1 = __float_as_uint(a0.y) & 0x7fffffffu;
    e[0] = (int)(b0 >> 23) - 126;
    e[1] = (int)(b1 >> 23) - 126;
    x = make_float2(__uint_as_float((b0 & 0x007fffffu) | 0x3f000000u), __uint_as_float((b1 & 0x007fffffu) | 0x3f000000u));
  } else {
    x = make_float2(math::pow_frexp(fabsf(a0.x), e[0]), math::pow_frexp(fabsf(a0.y), e[1]));
  }
  i[0] = math::pow_index(x.x);
  i[1] = math::pow_index(x.y);
  const float2 tmp = make_float2(math::pow_a(x.x, i[0]), math::pow_a(x.y, i[1]));
  x = sub(x, tmp);
  x = sub(x, make_float2(math::pow_b(x.x, i[0] >> 1), math::pow_b(x.y, i[1] >> 1)));
  x = markstein_quot(x, tmp);
  float2 z = mul(x, x);
  float2 w = mul_r(mul(z, x), horner<F>(x, P1));
  w = madd<F>(splat(-0.5f), z, w);
  w = madd<F>(splat(C::bits(C::log2_em1)), w, w);
  z = madd<F>(splat(C::bits(C::log2_em1)), x, w);
  z = add(z, x);
  w = madd<F>(make_float2((float)(-i[0]), (float)(-i[1])), splat(0.0625f), make_float2((float)e[0], (float)e[1]));
  const float2 ya = pow_reduc(a1);
  const float2 yb = sub(a1, ya);
  float2 W = madd<F>(z, a1, mul_r(w, yb));
  float2 Wa = pow_reduc(W);
  float2 Wb = sub(W, Wa);
  W = madd<F>(w, ya, Wa);
  Wa = pow_reduc(W);
  const float2 u = sub(W, Wa);
  W = add(Wb, u);
  Wb = pow_reduc(W);
  w = mul(splat(16.0f), add(Wa, Wb));
  const float wl[2] = {w.x, w.y};
  bool inf_ret[2], zer_ret[2];
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    inf_ret[l] = wl[l] > C::bits(C::large);
    zer_ret[l] = wl[l] < C::bits(C::low);
    e[l] = (int)fminf(fmaxf(wl[l], -32768.0f), 32768.0f);   // as math::pow_abs
  }
  Wb = sub(W, Wb);
  const bool t0 = Wb.x > 0.0f, t1 = Wb.y > 0.0f;
  e[0] = t0 ? e[0] + 1 : e[0];
  e[1] = t1 ? e[1] + 1 : e[1];
  const float2 Wm = sub(Wb, splat(0.0625f));
  Wb = make_float2(t0 ? Wm.x : Wb.x, t1 ? Wm.y : Wb.y);
  z = mul(horner<F>(Wb, P2), Wb);
  float wt[2];
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    i[l] = (e[l] > 0) ? e[l] / 16 + 1 : e[l] / 16;
    e[l] = i[l] * 16 - e[l];
    wt[l] = math::pow_a(0.0f, min(max(e[l], 0), 16));
  }
  w = make_float2(wt[0], wt[1]);
  z = madd<F>(w, z, w);
  z = pow_ldexp(z, i[0], i[1]);
  if constexpr (PLAIN) {
    const float inf = __int_as_float(0x7f800000);
    z.x = inf_ret[0] ? inf : (zer_ret[0] ? 0.0f : z.x);
    z.y = inf_ret[1] ? inf : (zer_ret[1] ? 0.0f : z.y);
    z.x = (fabsf(a0.x) == 1.0f) ? 1.0f : z.x;
    z.y = (fabsf(a0.y) == 1.0f) ? 1.0f : z.y;
    return z;
  } else {
    return make_float2(pow_special(a0.x, a1.x, z.x, zer_ret[0], inf_ret[0]),
                       pow_special(a0.y, a1.y, z.y, zer_ret[1], inf_ret[1]));
  }
}

// |a0| normal and finite, a1 finite (pos: a0 also positive, where pow is pow_abs)
__device__ __forceinline__ bool pow_plain(float a0, float a1, bool pos)
{
  const uint32_t b = pos ? __float_as_uint(a0) : (__float_as_uint(a0) & 0x7fffffffu);
  return b - 0x00800000u < 0x7f000000u && fabsf(a1) < __int_as_float(0x7f800000);
}

template <bool F> __device__ __forceinline__ float2 pow_abs(float2 a0, float2 a1)
{
  if (__all_sync(__activemask(), pow_plain(a0.x, a1.x, false) && pow_plain(a0.y, a1.y, false)))
    return pow_abs_core<F, true>(a0, a1);
  return pow_abs_core<F, false>(a0, a1);
}

template <bool F> __device__ __forceinline__ float2 pow(float2 a0, float2 a1)
{
  if (__all_sync(__activemask(), pow_plain(a0.x, a1.x, true) && pow_plain(a0.y, a1.y, true)))
    return pow_abs_core<F, true>(a0, a1);
  float2 z = pow_abs_core<F, false>(a0, a1);
  const float2 h = mul(sub(a1, splat(1.0f)), splat(0.5f));   // exact: a1 - 1 is 0 or normal
  const float al0[2] = {a0.x, a0.y}, al1[2] = {a1.x, a1.y}, hl[2] = {h.x, h.y};
  float zl[2] = {z.x, z.y};
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    const bool ltz = al0[l] < 0.0f;
    if (ltz && math::is_flint(hl[l])) zl[l] = -zl[l];
    zl[l] = (ltz && !math::is_flint(al1[l])) ? float(NAN) : zl[l];
  }
  return make_float2(zl[0], zl[1]);
}

// ------------------------------------------------------------------ cbrt
// NT2's float cbrt (math::cbrt), two lanes: the exponent split, the table
// factor and the special cases per lane, the polynomial and the Newton step
// packed.  The Newton step's division z / x^2 is markstein_quot when every
// lane of the warp has z >= 2^-103 (or z not finite): with a quotient of
// about z^(1/3), the residual z - x^2 q is then a multiple of at least
// 2^-149, so it is exact and the correction holds as it does for normal
// operands.  Other warps divide per lane.  Checked against the one-lane form
// over every float.
template <bool F> __device__ __forceinline__ float2 cbrt(float2 a0)
{
  constexpr uint32_t P[5] = {0xbe09e49au, 0x3f0bf0feu, 0xbf745265u, 0x3f91eb77u, 0x3ece0609u};
  const float al[2] = {a0.x, a0.y};
  float zl[2], fl[2], xl[2], factl[2], scl[2];
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    float z = fabsf(al[l]);
    const bool den = z < fbits(0x00800000u);
    z = den ? math::mul(z, 8388608.0f) : z;
    fl[l] = den ? fbits(0x3ba14518u) : 1.0f;   // 2^(-23/3)
    const uint32_t b = __float_as_uint(z);
    int e = (int)((b & 0x7f800000u) >> 23) - 126;
    xl[l] = fbits((b & ~0x7f800000u) | 0x3f000000u);
    const bool flag = e >= 0;
    int rem;
    e = math::cbrt_split(e, rem);
    float fact = rem == 1 ? (flag ? fbits(0x3fa14518u) : fbits(0x3f4b2ff5u)) : 1.0f;
    factl[l] = rem == 2 ? (flag ? fbits(0x3fcb2ff5u) : fbits(0x3f214518u)) : fact;
    scl[l] = fbits((uint32_t)(e + 127) << 23);
    zl[l] = z;
  }
  const float2 z = make_float2(zl[0], zl[1]);
  float2 x = horner<F>(make_float2(xl[0], xl[1]), P);
  x = mul_r(mul(x, make_float2(factl[0], factl[1])), make_float2(scl[0], scl[1]));
  const float2 xx = mul(x, x);
  const bool safe0 = !(zl[0] < fbits(0x0c000000u)), safe1 = !(zl[1] < fbits(0x0c000000u));   // 2^-103
  float2 q;
  if (__all_sync(__activemask(), safe0 && safe1)) q = markstein_quot(z, xx);
  else q = make_float2(__fdiv_rn(z.x, xx.x), __fdiv_rn(z.y, xx.y));
  x = sub(x, mul_r(sub(x, q), splat(fbits(0x3eaaaaabu))));
  x = mul(make_float2(__uint_as_float(__float_as_uint(x.x) | (__float_as_uint(a0.x) & 0x80000000u)),
                      __uint_as_float(__float_as_uint(x.y) | (__float_as_uint(a0.y) & 0x80000000u))),
          make_float2(fl[0], fl[1]));
  return make_float2((a0.x == 0.0f || isinf(a0.x)) ? a0.x : x.x, (a0.y == 0.0f || isinf(a0.y)) ? a0.y : x.y);
}

}  // namespace x2
}  // namespace nt2cuda
