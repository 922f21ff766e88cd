// nt2cuda/trig.cuh -- NT2's sin, cos, tan (radians) and sinpi, cospi for
// float and double, evaluated over packs of lanes the way NT2's SIMD
// transform evaluates them.
//
// Paths are relative to NT2's modules/core/trigonometric/include/nt2/trigonometric/.
//
// NT2 reduces a whole pack with one method, chosen from the pack's largest
// |x| (functions/scalar/impl/trigo/trig_reduction.hpp:46-183, mode big_ of
// functions/scalar/impl/selection_tags.hpp:55-61):
//   level 0  all |x| <= pi/4       no reduction
//   level 1  all |x| <= pi/2       rem_pio2_straight   (functions/generic/rem_pio2_straight.hpp)
//   level 2  all |x| <= 20 pi      rem_pio2_cephes     (functions/generic/rem_pio2_cephes.hpp)
//   level 3  all |x| <= Medium_pi  rem_pio2_medium     (functions/generic/rem_pio2_medium.hpp);
//                                  Medium_pi = 2^6 pi (float), 2^18 pi (double)
//   level 4  float, all |x| <= 2^18 pi: each half pack converted to double and
//            reduced by the double chain
//   level 5  rem_pio2 lane by lane (functions/scalar/rem_pio2.hpp, fdlibm)
// one() is NT2's scalar code (each element its own pack); pack<P>() is NT2's
// SIMD code over P lanes, used with P = one 16-byte group of a thread (4
// floats, 2 doubles: NT2 on a 128-bit SIMD extension).
// Lanes that reach fdlibm's __kernel_rem_pio2(f) (float |x| > 2^7 pi/2 at level
// 5, double |x| > 2^19 pi/2) use an exact Payne-Hanek reduction rounded once.
// The polynomials are functions/simd/common/impl/trigo/{f,d}_trig_evaluation.hpp
// with NT2's unfused fma; F (fused) contracts them.
#pragma once
#include <stdint.h>
#include <type_traits>
#include "bs_x2.cuh"
#include "math.cuh"

namespace nt2cuda {
namespace trig {

using math::fbits;
using math::dbits;

enum kind { SIN = 0, COS = 1, TAN = 2, SINPI = 3, COSPI = 4, COT = 5, TANPI = 6, COTPI = 7, SIND = 8, COSD = 9,
            TAND = 10, COTD = 11 };
// the reduction a kind takes: pi_tag (x in half turns), degree_tag, or radians (pack-level method)
__host__ __device__ constexpr bool pi_kind(int k) { return k == SINPI || k == COSPI || k == TANPI || k == COTPI; }
__host__ __device__ constexpr bool deg_kind(int k) { return k >= SIND && k <= COTD; }

// Bit patterns of the BOOST_SIMD_CONSTANT_REGISTER lines in constants/*.hpp.
struct tf {
  static constexpr uint32_t pio4 = 0x3f490fdbu, pio2 = 0x3fc90fdbu, p20pi = 0x427b53d1u,
                            medpi = 0x43490fdbu, dmpi = 0x49490fdbu, pi = 0x40490fdbu,
                            twoopi = 0x3f22f983u, invpio2 = 0x3f22f984u, pio2_1 = 0x3fc90f80u,
                            pio2_2 = 0x37354400u, pio2_3 = 0x2e85a300u, pio2_1t = 0x37354443u,
                            pio2_2t = 0x2e85a308u, pio2_3t = 0x248d3132u;
};
struct td {
  static constexpr uint64_t pio4 = 0x3fe921fb54442d18ull, pio2 = 0x3ff921fb54442d18ull,
                            p20pi = 0x404f6a7a2955385eull, medpi = 0x412921fb54442d18ull,
                            pi = 0x400921fb54442d18ull, twoopi = 0x3fe45f306dc9c883ull,
                            invpio2 = 0x3fe45f306dc9c883ull, pio2_1 = 0x3ff921fb54400000ull,
                            pio2_2 = 0x3dd0b4611a600000ull, pio2_3 = 0x3ba3198a2e000000ull,
                            pio2_1t = 0x3dd0b4611a626331ull, pio2_2t = 0x3ba3198a2e037073ull,
                            pio2_3t = 0x397b839a252049c1ull;
};

// High bits of n*pi/2, n = 1..32 (float: pattern with the low 8 bits
// cleared; double: high word): the cancellation test of fdlibm's medium branch.
__device__ __constant__ const uint32_t kNpio2F[32] = {
  0x3fc90f00u, 0x40490f00u, 0x4096cb00u, 0x40c90f00u, 0x40fb5300u, 0x4116cb00u, 0x412fed00u, 0x41490f00u,
  0x41623100u, 0x417b5300u, 0x418a3a00u, 0x4196cb00u, 0x41a35c00u, 0x41afed00u, 0x41bc7e00u, 0x41c90f00u,
  0x41d5a000u, 0x41e23100u, 0x41eec200u, 0x41fb5300u, 0x4203f200u, 0x420a3a00u, 0x42108300u, 0x4216cb00u,
  0x421d1400u, 0x42235c00u, 0x4229a500u, 0x422fed00u, 0x42363600u, 0x423c7e00u, 0x4242c700u, 0x42490f00u};
__device__ __constant__ const uint32_t kNpio2D[32] = {
  0x3ff921fbu, 0x400921fbu, 0x4012d97cu, 0x401921fbu, 0x401f6a7au, 0x4022d97cu, 0x4025fdbbu, 0x402921fbu,
  0x402c463au, 0x402f6a7au, 0x4031475cu, 0x4032d97cu, 0x40346b9cu, 0x4035fdbbu, 0x40378fdbu, 0x403921fbu,
  0x403ab41bu, 0x403c463au, 0x403dd85au, 0x403f6a7au, 0x40407e4cu, 0x4041475cu, 0x4042106cu, 0x4042d97cu,
  0x4043a28cu, 0x40446b9cu, 0x404534acu, 0x4045fdbbu, 0x4046c6cbu, 0x40478fdbu, 0x404858ebu, 0x404921fbu};

// 2/pi, bits after the binary point, 32 per word.
__device__ __constant__ const uint32_t kTwoOverPi[40] = {
  0xa2f9836eu, 0x4e441529u, 0xfc2757d1u, 0xf534ddc0u, 0xdb629599u, 0x3c439041u, 0xfe5163abu, 0xdebbc561u,
  0xb7246e3au, 0x424dd2e0u, 0x06492eeau, 0x09d1921cu, 0xfe1deb1cu, 0xb129a73eu, 0xe88235f5u, 0x2ebb4484u,
  0xe99c7026u, 0xb45f7e41u, 0x3991d639u, 0x835339f4u, 0x9c845f8bu, 0xbdf9283bu, 0x1ff897ffu, 0xde05980fu,
  0xef2f118bu, 0x5a0a6d1fu, 0x6d367ecfu, 0x27cb09b7u, 0x4f463f66u, 0x9e5fea2du, 0x7527bac7u, 0xebe5f17bu,
  0x3d0739f7u, 0x8a5292eau, 0x6bfb5fb1u, 0x1f8d5d08u, 0x56033046u, 0xfc7b6babu, 0xf0cfbc20u, 0x9af4361du};

// A reduced argument: x - n*pi/2 and n mod 4.  Returned by value, so that the
// out-of-line reductions below take no address of the caller's registers.
template <class T> struct reduced { T xr; int n; };

// ------------------------------------------------ exact Payne-Hanek reduction
// 64-bit limbs, little-endian.
template <int N> __device__ __forceinline__ int lbit(const uint64_t (&p)[N], int k)
{
  return (k < 0 || k >= 64 * N) ? 0 : (int)((p[k >> 6] >> (k & 63)) & 1ull);
}
template <int N> __device__ __forceinline__ uint64_t lword(const uint64_t (&p)[N], int i)
{
  return (i < 0 || i >= N) ? 0ull : p[i];
}
// bits [k, k + 64)
template <int N> __device__ __forceinline__ uint64_t lbits64(const uint64_t (&p)[N], int k)
{
  const int i = k >= 0 ? (k >> 6) : -((-k + 63) >> 6);
  const int s = k - 64 * i;
  const uint64_t lo = lword(p, i), hi = lword(p, i + 1);
  return s == 0 ? lo : ((lo >> s) | (hi << (64 - s)));
}
// any bit in [0, k)
template <int N> __device__ __forceinline__ bool lany_below(const uint64_t (&p)[N], int k)
{
  for (int i = 0; i < N; ++i) {
    const int lo = 64 * i;
    if (lo >= k) break;
    const uint64_t m = (k - lo >= 64) ? ~0ull : ((1ull << (k - lo)) - 1ull);
    if (p[i] & m) return true;
  }
  return false;
}

// x = m * 2^q (m < 2^53, x > 0 finite): n = round(x * 2/pi) mod 4 and
// r = x - n*pi/2, rounded once to `prec` bits.  A 256-bit window of 2/pi
// starting at the first word that can reach the integer part mod 4.
static __device__ __noinline__ reduced<double> exact_rem_pio2(uint64_t m, int q, int prec)
{
  const int i0 = q >= 2 ? (q - 2) / 32 : 0;
  uint64_t nw[4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
    nw[3 - j] = ((uint64_t)kTwoOverPi[i0 + 2 * j] << 32) | kTwoOverPi[i0 + 2 * j + 1];
  uint64_t p[5];
  uint64_t c = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint64_t lo = m * nw[j];
    uint64_t hi = __umul64hi(m, nw[j]);
    lo += c;
    hi += (lo < c) ? 1ull : 0ull;
    p[j] = lo;
    c = hi;
  }
  p[4] = c;
  const int sh = 32 * (i0 + 8) - q;          // fraction bits of p (223..301)
  int n = lbit(p, sh) | (lbit(p, sh + 1) << 1);
#pragma unroll
  for (int i = 0; i < 5; ++i) {               // keep the fraction
    const int lo = 64 * i;
    p[i] = lo >= sh ? 0ull : ((sh - lo >= 64) ? p[i] : (p[i] & ((1ull << (sh - lo)) - 1ull)));
  }
  const bool neg = lbit(p, sh - 1) != 0;
  if (neg) {                                  // p = 2^sh - p = (-p) mod 2^sh, n = n + 1
    n += 1;
    uint64_t cc = 1;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int lo = 64 * i;
      const uint64_t mask = lo >= sh ? 0ull : ((sh - lo >= 64) ? ~0ull : ((1ull << (sh - lo)) - 1ull));
      const uint64_t v = ~p[i] + cc;
      cc = (cc != 0ull && v == 0ull) ? 1ull : 0ull;
      p[i] = v & mask;
    }
  }
  int top = -1;
  for (int i = 4; i >= 0; --i)
    if (p[i]) { top = 64 * i + 63 - __clzll((long long)p[i]); break; }
  if (top < 0) return reduced<double>{0.0, n & 3};
  const uint64_t mh = lbits64(p, top - 63), ml = lbits64(p, top - 127);
  const bool sticky_f = lany_below(p, top - 127);
  // Q = M * floor(pi/2 * 2^126)
  const uint64_t ph = 0x6487ed5110b4611aull, pl = 0x62633145c06e0e68ull;
  uint64_t Q[4];
  {
    const uint64_t a0 = ml * pl, a1 = __umul64hi(ml, pl);
    const uint64_t b0 = ml * ph, b1 = __umul64hi(ml, ph);
    const uint64_t c0 = mh * pl, c1 = __umul64hi(mh, pl);
    const uint64_t d0 = mh * ph, d1 = __umul64hi(mh, ph);
    Q[0] = a0;
    uint64_t s1 = a1 + b0;
    uint64_t k1 = s1 < a1 ? 1ull : 0ull;
    const uint64_t t1 = s1 + c0;
    k1 += t1 < s1 ? 1ull : 0ull;
    Q[1] = t1;
    uint64_t s2 = b1 + c1;
    uint64_t k2 = s2 < b1 ? 1ull : 0ull;
    const uint64_t t2 = s2 + d0;
    k2 += t2 < s2 ? 1ull : 0ull;
    const uint64_t u2 = t2 + k1;
    k2 += u2 < t2 ? 1ull : 0ull;
    Q[2] = u2;
    Q[3] = d1 + k2;
  }
  const int T = lbit(Q, 254) ? 254 : 253;
  const uint64_t mant = lbits64(Q, T - 63);
  const bool sticky = sticky_f || lany_below(Q, T - 63);
  const int drop = 64 - prec;
  uint64_t mm = mant >> drop;
  const uint64_t rem = mant & ((1ull << drop) - 1ull), half = 1ull << (drop - 1);
  int e = (T - 63) + (top - 253 - sh) + drop;
  if (rem > half || (rem == half && (sticky || (mm & 1ull)))) ++mm;
  if (mm >> prec) { mm >>= 1; ++e; }
  // mm * 2^e, a normal double: |r| lies in [2^-70, pi/4]
  const int be = e + prec - 1 + 1023;
  const uint64_t bits = ((uint64_t)be << 52) | ((mm << (53 - prec)) & 0xfffffffffffffull);
  const double v = __longlong_as_double((long long)bits);
  return reduced<double>{neg ? -v : v, n & 3};
}

// -------------------------------------------------------------- reductions
// cvttps2dq / cvttpd2dq: NaN or out of range gives INT32_MIN (a plain cast
// saturates instead).  A float overload keeps float code off the FP64 pipe.
__device__ __forceinline__ int toint32(float a)
{
  return (a != a || a >= 2147483648.0f || a < -2147483648.0f) ? (int)0x80000000 : (int)a;
}
__device__ __forceinline__ int toint32(double a)
{
  return (a != a || a >= 2147483648.0 || a < -2147483648.0) ? (int)0x80000000 : (int)a;
}
__device__ __forceinline__ long long toint64(double a)
{
  return (a != a || a >= 9223372036854775808.0 || a < -9223372036854775808.0) ? (long long)0x8000000000000000ull
                                                                               : (long long)a;
}

__device__ __forceinline__ int straight(float x, float& xr)
{
  float r = __fsub_rn(x, fbits(tf::pio2_1));
  r = __fsub_rn(r, fbits(tf::pio2_2));
  xr = __fsub_rn(r, fbits(tf::pio2_3));
  return 1;
}
__device__ __forceinline__ int straight(double x, double& xr)
{
  double r = __dsub_rn(x, dbits(td::pio2_1));
  r = __dsub_rn(r, dbits(td::pio2_2));
  xr = __dsub_rn(r, dbits(td::pio2_3));
  return 1;
}
__device__ __forceinline__ int cephes(float x, float& xr)
{
  const float xi = rintf(__fmul_rn(x, fbits(tf::twoopi)));
  float r = __fsub_rn(x, __fmul_rn(xi, fbits(tf::pio2_1)));
  r = __fsub_rn(r, __fmul_rn(xi, fbits(tf::pio2_2)));
  xr = __fsub_rn(r, __fmul_rn(xi, fbits(tf::pio2_3)));
  return (int)xi & 3;     // |xi| <= 40 (or NaN, whose xr is NaN whatever n is)
}
__device__ __forceinline__ int cephes(double x, double& xr)
{
  const double xi = rint(__dmul_rn(x, dbits(td::twoopi)));
  double r = __dsub_rn(x, __dmul_rn(xi, dbits(td::pio2_1)));
  r = __dsub_rn(r, __dmul_rn(xi, dbits(td::pio2_2)));
  xr = __dsub_rn(r, __dmul_rn(xi, dbits(td::pio2_3)));
  return (int)xi & 3;     // |xi| <= 40 (or NaN, whose xr is NaN whatever n is)
}
template <class T, class C> __device__ __forceinline__ int medium_impl(T t, T& xr, T invpio2, T p1, T p2, T p2t, T p3, T p3t)
{
  using math::add; using math::sub; using math::mul;
  const T fn = C::round(mul(t, invpio2));
  T r = sub(t, mul(fn, p1));
  T t2 = r, w = mul(fn, p2);
  r = sub(t2, w);
  w = sub(mul(fn, p2t), sub(sub(t2, r), w));
  t2 = r;
  w = mul(fn, p3);
  r = sub(t2, w);
  w = sub(mul(fn, p3t), sub(sub(t2, r), w));
  xr = sub(r, w);
  return C::toint(fn) & 3;
}
// medium's quotients are below 2^7 (float) and 2^19 (double), or NaN
struct cvt_f { __device__ static float round(float a) { return rintf(a); } __device__ static int toint(float a) { return (int)a; } };
struct cvt_d { __device__ static double round(double a) { return rint(a); } __device__ static int toint(double a) { return (int)a; } };
__device__ __forceinline__ int medium(float t, float& xr)
{
  return medium_impl<float, cvt_f>(t, xr, fbits(tf::invpio2), fbits(tf::pio2_1), fbits(tf::pio2_2), fbits(tf::pio2_2t),
                                   fbits(tf::pio2_3), fbits(tf::pio2_3t));
}
__device__ __forceinline__ int medium(double t, double& xr)
{
  return medium_impl<double, cvt_d>(t, xr, dbits(td::invpio2), dbits(td::pio2_1), dbits(td::pio2_2), dbits(td::pio2_2t),
                                    dbits(td::pio2_3), dbits(td::pio2_3t));
}

// fdlibm __ieee754_rem_pio2f for x >= 0 (functions/scalar/rem_pio2.hpp:148-231)
static __device__ __noinline__ reduced<float> fdlibm(float x)
{
  const uint32_t ix = __float_as_uint(x) & 0x7fffffffu;
  float xr;
  int n;
  if (ix <= 0x3f490fd8u) {
    xr = x; n = 0;
  } else if (ix < 0x4016cbe4u) {
    float z = __fsub_rn(x, fbits(tf::pio2_1));
    if ((ix & 0xfffffff0u) != 0x3fc90fd0u) {
      xr = __fsub_rn(z, fbits(tf::pio2_1t));
    } else {
      z = __fsub_rn(z, fbits(tf::pio2_2));
      xr = __fsub_rn(z, fbits(tf::pio2_2t));
    }
    n = 1;
  } else if (ix <= 0x43490f80u) {
    const int ni = (int)__fadd_rn(__fmul_rn(x, fbits(tf::invpio2)), 0.5f);
    const float fn = (float)ni;
    float r = __fsub_rn(x, __fmul_rn(fn, fbits(tf::pio2_1)));
    float w = __fmul_rn(fn, fbits(tf::pio2_1t));
    float y0 = __fsub_rn(r, w);
    if (!(ni < 32 && (ix & 0xffffff00u) != kNpio2F[ni - 1])) {
      const int j = (int)(ix >> 23);
      int i = j - (int)((__float_as_uint(y0) >> 23) & 0xffu);
      if (i > 8) {
        float t = r;
        w = __fmul_rn(fn, fbits(tf::pio2_2));
        r = __fsub_rn(t, w);
        w = __fsub_rn(__fmul_rn(fn, fbits(tf::pio2_2t)), __fsub_rn(__fsub_rn(t, r), w));
        y0 = __fsub_rn(r, w);
        i = j - (int)((__float_as_uint(y0) >> 23) & 0xffu);
        if (i > 25) {
          t = r;
          w = __fmul_rn(fn, fbits(tf::pio2_3));
          r = __fsub_rn(t, w);
          w = __fsub_rn(__fmul_rn(fn, fbits(tf::pio2_3t)), __fsub_rn(__fsub_rn(t, r), w));
          y0 = __fsub_rn(r, w);
        }
      }
    }
    xr = y0;
    n = ni & 3;
  } else if (ix >= 0x7f800000u) {
    xr = __fsub_rn(x, x); n = 0;
  } else {
    const reduced<double> e = exact_rem_pio2((uint64_t)((ix & 0x7fffffu) | 0x800000u), (int)(ix >> 23) - 150, 24);
    xr = (float)e.xr;
    n = e.n;
  }
  return {xr, n};
}

// NT2's double rem_pio2 (functions/scalar/rem_pio2.hpp:413-427) over fdlibm
// __ieee754_rem_pio2 for x >= 0 (:536-621)
static __device__ __noinline__ reduced<double> fdlibm(double x)
{
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t ix = (uint32_t)(b >> 32) & 0x7fffffffu;
  double xr;
  int n;
  if (b == 0x7ff0000000000000ull) {
    xr = __longlong_as_double(0x7ff8000000000000ll); n = 0;
  } else if (ix <= 0x3fe921fbu) {
    xr = x; n = 0;
  } else if (ix < 0x4002d97cu) {
    double z = __dsub_rn(x, dbits(td::pio2_1));
    if (ix != 0x3ff921fbu) {
      xr = __dsub_rn(z, dbits(td::pio2_1t));
    } else {
      z = __dsub_rn(z, dbits(td::pio2_2));
      xr = __dsub_rn(z, dbits(td::pio2_2t));
    }
    n = 1;
  } else if (ix <= 0x413921fbu) {
    const int ni = (int)__dadd_rn(__dmul_rn(x, dbits(td::invpio2)), 0.5);
    const double fn = (double)ni;
    double r = __dsub_rn(x, __dmul_rn(fn, dbits(td::pio2_1)));
    double w = __dmul_rn(fn, dbits(td::pio2_1t));
    double y0 = __dsub_rn(r, w);
    if (!(ni < 32 && ni > 0 && ix != kNpio2D[ni - 1])) {
      const int j = (int)(ix >> 20);
      int i = j - (int)(((uint64_t)__double_as_longlong(y0) >> 52) & 0x7ffu);
      if (i > 16) {
        double t = r;
        w = __dmul_rn(fn, dbits(td::pio2_2));
        r = __dsub_rn(t, w);
        w = __dsub_rn(__dmul_rn(fn, dbits(td::pio2_2t)), __dsub_rn(__dsub_rn(t, r), w));
        y0 = __dsub_rn(r, w);
        i = j - (int)(((uint64_t)__double_as_longlong(y0) >> 52) & 0x7ffu);
        if (i > 49) {
          t = r;
          w = __dmul_rn(fn, dbits(td::pio2_3));
          r = __dsub_rn(t, w);
          w = __dsub_rn(__dmul_rn(fn, dbits(td::pio2_3t)), __dsub_rn(__dsub_rn(t, r), w));
          y0 = __dsub_rn(r, w);
        }
      }
    }
    xr = y0;
    n = ni & 3;
  } else if (ix >= 0x7ff00000u) {
    xr = __dsub_rn(x, x); n = 0;
  } else {
    const reduced<double> e = exact_rem_pio2((b & 0xfffffffffffffull) | (1ull << 52), (int)((b >> 52) & 0x7ffu) - 1075, 53);
    xr = e.xr;
    n = e.n;
  }
  return {xr, n};
}

// Level of a lane: how many thresholds |x| exceeds (NaN: 0).
__device__ __forceinline__ int level(float x)
{
  return (x > fbits(tf::pio4)) + (x > fbits(tf::pio2)) + (x > fbits(tf::p20pi)) + (x > fbits(tf::medpi)) +
         (x > fbits(tf::dmpi));
}
__device__ __forceinline__ int level(double x)
{
  return (x > dbits(td::pio4)) + (x > dbits(td::pio2)) + (x > dbits(td::p20pi)) + (x > dbits(td::medpi));
}

// Largest |x| of a pack (NaN lanes ignored, as their level is 0); level() is
// monotone, so the pack's level is the level of its largest lane.
template <int P, class T> __device__ __forceinline__ T pack_max(const T (&x)[P])
{
  T m = x[0];
#pragma unroll
  for (int l = 1; l < P; ++l) m = fmax(m, x[l]);
  return m;
}

// The double chain over one pack of P lanes at level lv.
template <int P> __device__ __forceinline__ void reduce_at(int lv, const double (&x)[P], double (&xr)[P], int (&n)[P])
{
  if (lv == 0) {
#pragma unroll
    for (int l = 0; l < P; ++l) { xr[l] = x[l]; n[l] = 0; }
  } else if (lv == 1) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = straight(x[l], xr[l]);
  } else if (lv == 2) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = cephes(x[l], xr[l]);
  } else if (lv == 3) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = medium(x[l], xr[l]);
  } else {
#pragma unroll
    for (int l = 0; l < P; ++l) { const auto r = fdlibm(x[l]); xr[l] = r.xr; n[l] = r.n; }
  }
}
template <int P> __device__ __forceinline__ void reduce_pack(const double (&x)[P], double (&xr)[P], int (&n)[P])
{
  reduce_at<P>(level(pack_max<P>(x)), x, xr, n);
}

// The float chain over one pack of P lanes at level lv.
template <int P> __device__ __forceinline__ void reduce_at(int lv, const float (&x)[P], float (&xr)[P], int (&n)[P])
{
  if (lv == 0) {
#pragma unroll
    for (int l = 0; l < P; ++l) { xr[l] = x[l]; n[l] = 0; }
  } else if (lv == 1) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = straight(x[l], xr[l]);
  } else if (lv == 2) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = cephes(x[l], xr[l]);
  } else if (lv == 3) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = medium(x[l], xr[l]);
  } else if (lv == 4) {
    // halves of the pack through the double chain
    constexpr int H = P > 1 ? P / 2 : 1;
#pragma unroll
    for (int s = 0; s < P; s += H) {
      double xd[H], rd[H];
      int nd[H];
#pragma unroll
      for (int l = 0; l < H; ++l) xd[l] = (double)x[s + l];
      reduce_pack<H>(xd, rd, nd);
#pragma unroll
      for (int l = 0; l < H; ++l) { xr[s + l] = (float)rd[l]; n[s + l] = nd[l]; }
    }
  } else {
#pragma unroll
    for (int l = 0; l < P; ++l) { const auto r = fdlibm(x[l]); xr[l] = r.xr; n[l] = r.n; }
  }
}
template <int P> __device__ __forceinline__ void reduce_pack(const float (&x)[P], float (&xr)[P], int (&n)[P])
{
  reduce_at<P>(level(pack_max<P>(x)), x, xr, n);
}

// pi_tag reduction (trig_reduction.hpp:216-229): xi = round2even(2x),
// xr = (x - xi/2) * pi, n = fast_toint(xi).
__device__ __forceinline__ int reduce_pi(float x, float& xr, bool)
{
  const float xi = rintf(__fmul_rn(x, 2.0f));
  xr = __fmul_rn(__fsub_rn(x, __fmul_rn(xi, 0.5f)), fbits(tf::pi));
  return toint32(xi) & 3;
}
__device__ __forceinline__ int reduce_pi(double x, double& xr, bool simd)
{
  const double xi = rint(__dmul_rn(x, 2.0));
  xr = __dmul_rn(__dsub_rn(x, __dmul_rn(xi, 0.5)), dbits(td::pi));
  // SSE2 converts packed doubles through int32 (cvttpd2dq); scalar code casts to int64
  return simd ? (toint32(xi) & 3) : (int)(toint64(xi) & 3);
}

// degree_tag reduction (trig_reduction.hpp:262-278, the form without x87):
// xi = round2even(x/90), xr = inrad(x - xi*90), n = fast_toint(xi), converted
// as the pi_tag reduction converts it.
__device__ __forceinline__ int reduce_deg(float x, float& xr, bool)
{
  const float xi = rintf(__fmul_rn(x, fbits(0x3c360b61u)));
  xr = __fmul_rn(__fsub_rn(x, __fmul_rn(xi, 90.0f)), fbits(0x3c8efa35u));
  return toint32(xi) & 3;
}
__device__ __forceinline__ int reduce_deg(double x, double& xr, bool simd)
{
  const double xi = rint(__dmul_rn(x, dbits(0x3f86c16c16c16c17ull)));
  xr = __dmul_rn(__dsub_rn(x, __dmul_rn(xi, 90.0)), dbits(0x3f91df46a2529d39ull));
  return simd ? (toint32(xi) & 3) : (int)(toint64(xi) & 3);
}
template <int K, class T> __device__ __forceinline__ int reduce_unit(T x, T& xr, bool simd)
{
  if constexpr (pi_kind(K)) return reduce_pi(x, xr, simd);
  else return reduce_deg(x, xr, simd);
}

// ------------------------------------------------------------- evaluation
// functions/simd/common/impl/trigo/f_trig_evaluation.hpp:25-56
template <bool F> __device__ __forceinline__ float cos_eval(float z)
{
  constexpr uint32_t C[3] = {0x37ccf5ceu, 0xbab60619u, 0x3d2aaaa5u};
  const float y = math::horner<F>(z, C);
  return __fadd_rn(1.0f, math::madd<F>(z, -0.5f, __fmul_rn(y, __fmul_rn(z, z))));
}
template <bool F> __device__ __forceinline__ float sin_eval(float z, float x)
{
  constexpr uint32_t C[3] = {0xb94ca1f9u, 0x3c08839du, 0xbe2aaaa2u};
  return math::madd<F>(__fmul_rn(math::horner<F>(z, C), z), x, x);
}
template <bool F> __device__ __forceinline__ float tan_eval(float x)
{
  constexpr uint32_t C[6] = {0x3c19c53bu, 0x3b4c779cu, 0x3cc821b5u, 0x3d5ac5c9u, 0x3e0896ddu, 0x3eaaaa6fu};
  const float zz = __fmul_rn(x, x);
  return math::madd<F>(__fmul_rn(math::horner<F>(zz, C), zz), x, x);
}
// functions/simd/common/impl/trigo/d_trig_evaluation.hpp:25-66
template <bool F> __device__ __forceinline__ double cos_eval(double z)
{
  constexpr uint64_t C[7] = {0x3da8ff831ad9b219ull, 0xbe21eea7c1e514d4ull, 0x3e927e4f8e06d9a5ull,
                             0xbefa01a019ddbcd9ull, 0x3f56c16c16c15d47ull, 0xbfa5555555555551ull,
                             0x3fe0000000000000ull};
  return math::nmsub<F>(math::horner<F>(z, C), z, 1.0);
}
template <bool F> __device__ __forceinline__ double sin_eval(double z, double x)
{
  constexpr uint64_t C[6] = {0x3de5d8fd1fcf0ec1ull, 0xbe5ae5e5a9291691ull, 0x3ec71de3567d4896ull,
                             0xbf2a01a019bfdf03ull, 0x3f8111111110f7d0ull, 0xbfc5555555555548ull};
  return math::madd<F>(__dmul_rn(math::horner<F>(z, C), z), x, x);
}
template <bool F> __device__ __forceinline__ double tan_eval(double x)
{
  constexpr uint64_t N[3] = {0xc0c992d8d24f3f38ull, 0x413199eca5fc9dddull, 0xc1711fead3299176ull};
  constexpr uint64_t D[5] = {0x3ff0000000000000ull, 0x40cab8a5eeb36572ull, 0xc13427bc582abc96ull,
                             0x4177d98fc2ead8efull, 0xc189afe03cbe5a31ull};
  const double zz = __dmul_rn(x, x);
  const double q = __ddiv_rn(math::horner<F>(zz, N), math::horner<F>(zz, D));
  return math::madd<F>(x, __dmul_rn(zz, q), x);
}

template <class T> __device__ __forceinline__ T oneo_180();
template <> __device__ __forceinline__ float oneo_180<float>() { return fbits(0x3bb60b61u); }
template <> __device__ __forceinline__ double oneo_180<double>() { return dbits(0x3f76c16c16c16c17ull); }
__device__ __forceinline__ float flip(float v, uint32_t s) { return __uint_as_float(__float_as_uint(v) ^ s); }
__device__ __forceinline__ double flip(double v, uint64_t s)
{
  return __longlong_as_double((long long)((uint64_t)__double_as_longlong(v) ^ s));
}
__device__ __forceinline__ uint32_t sign_of(float a) { return __float_as_uint(a) & 0x80000000u; }
__device__ __forceinline__ uint64_t sign_of(double a) { return (uint64_t)__double_as_longlong(a) & 0x8000000000000000ull; }
template <class T> struct bits_of;
template <> struct bits_of<float> { using type = uint32_t; static constexpr int top = 31; };
template <> struct bits_of<double> { using type = uint64_t; static constexpr int top = 63; };

// NT2's invalid-argument tests of tana / cota per unit (scalar/impl/trigo/
// trig_reduction.hpp:89-90, 268-269, 308-309): none in radians; pi_tag: tan
// where x - 1/2 is an integer, cot at nonzero integers; degree_tag: tan where
// (x - 90)/180 is an integer, cot at nonzero multiples of 180.
template <int K, class T> __device__ __forceinline__ bool tan_invalid(T a0)
{
  if constexpr (K == TANPI) return math::is_flint(math::sub(a0, T(0.5)));
  else if constexpr (K == TAND) return math::is_flint(math::mul(math::sub(a0, T(90)), oneo_180<T>()));
  else return false;
}
template <int K, class T> __device__ __forceinline__ bool cot_invalid(T a0)
{
  if constexpr (K == COTPI) return a0 != T(0) && math::is_flint(a0);
  else if constexpr (K == COTD) return a0 != T(0) && math::is_flint(math::mul(a0, oneo_180<T>()));
  else return false;
}

// trig_base sina / cosa / tana / cota (functions/simd/common/impl/trigo/trig_base.hpp:72-141;
// cota of a zero is rec(a0), an infinity with its sign)
template <int K, bool F, class T> __device__ __forceinline__ T finish(T a0, T xr, int n)
{
  using U = typename bits_of<T>::type;
  constexpr int top = bits_of<T>::top;
  if constexpr (K == TAN || K == TANPI || K == TAND) {
    T y = tan_eval<F>(xr);
    if (n & 1) y = -math::div(T(1), y);
    y = flip(y, sign_of(a0));
    return tan_invalid<K>(a0) ? T(NAN) : y;
  } else if constexpr (K == COT || K == COTPI || K == COTD) {
    T y = tan_eval<F>(xr);
    y = (n & 1) ? -y : math::div(T(1), y);
    y = flip(y, sign_of(a0));
    y = cot_invalid<K>(a0) ? T(NAN) : y;
    return a0 != T(0) ? y : math::div(T(1), a0);
  } else {
    const T z = math::mul(xr, xr);
    if constexpr (K == SIN || K == SINPI || K == SIND) {
      const T v = (n & 1) ? cos_eval<F>(z) : sin_eval<F>(z, xr);
      return flip(v, sign_of(a0) ^ ((U)(n & 2) << (top - 1)));
    } else {
      const T v = (n & 1) ? sin_eval<F>(z, xr) : cos_eval<F>(z);
      return flip(v, (U)((n ^ (n >> 1)) & 1) << top);
    }
  }
}

// finish for two float lanes: for the sine and cosine kinds both polynomials
// (cos_eval, sin_eval), for the tangent and cotangent kinds tan_eval, on
// packed FP32 instructions (nt2cuda/bs_x2.cuh), then each lane's pick, sign
// and reciprocal as finish does; bit-identical to two finish calls (checked
// over every float by nt2cuda_selftest_x2).
template <int K> struct sincos_kind {
  static constexpr bool value = K == SIN || K == COS || K == SINPI || K == COSPI || K == SIND || K == COSD;
};
template <int K> struct tancot_kind {
  static constexpr bool value = K == TAN || K == TANPI || K == TAND || K == COT || K == COTPI || K == COTD;
};
template <int K, bool F>
__device__ __forceinline__ void finish2(float a0, float a1, float xr0, float xr1, int n0, int n1, float& y0, float& y1)
{
  if constexpr (tancot_kind<K>::value) {
    // tan_eval of both lanes packed, the rest of finish per lane
    constexpr uint32_t TC[6] = {0x3c19c53bu, 0x3b4c779cu, 0x3cc821b5u, 0x3d5ac5c9u, 0x3e0896ddu, 0x3eaaaa6fu};
    const float2 x = make_float2(xr0, xr1);
    const float2 zz = x2::mul(x, x);
    const float2 tv = x2::madd<F>(x2::mul(x2::horner<F>(zz, TC), zz), x, x);
    const float a[2] = {a0, a1}, t[2] = {tv.x, tv.y};
    const int n[2] = {n0, n1};
    float y[2];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      float v = t[l];
      if constexpr (K == TAN || K == TANPI || K == TAND) {
        if (n[l] & 1) v = -math::div(1.0f, v);
        v = flip(v, sign_of(a[l]));
        y[l] = tan_invalid<K>(a[l]) ? float(NAN) : v;
      } else {
        v = (n[l] & 1) ? -v : math::div(1.0f, v);
        v = flip(v, sign_of(a[l]));
        v = cot_invalid<K>(a[l]) ? float(NAN) : v;
        y[l] = a[l] != 0.0f ? v : math::div(1.0f, a[l]);
      }
    }
    y0 = y[0];
    y1 = y[1];
    return;
  }
  constexpr uint32_t CC[3] = {0x37ccf5ceu, 0xbab60619u, 0x3d2aaaa5u};
  constexpr uint32_t SC[3] = {0xb94ca1f9u, 0x3c08839du, 0xbe2aaaa2u};
  const float2 x = make_float2(xr0, xr1);
  const float2 z = x2::mul(x, x);
  // cos_eval: 1 + madd(z, -0.5, horner(z)*(z*z)); sin_eval: madd(horner(z)*z, x, x)
  const float2 cv = x2::add(x2::splat(1.0f),
                            x2::madd<F>(z, x2::splat(-0.5f), x2::mul_r(x2::horner<F>(z, CC), x2::mul(z, z))));
  const float2 sv = x2::madd<F>(x2::mul(x2::horner<F>(z, SC), z), x, x);
  const float a[2] = {a0, a1};
  const int n[2] = {n0, n1};
  const float c[2] = {cv.x, cv.y}, s[2] = {sv.x, sv.y};
  float y[2];
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    if constexpr (K == SIN || K == SINPI || K == SIND) {
      const float v = (n[l] & 1) ? c[l] : s[l];
      y[l] = flip(v, sign_of(a[l]) ^ ((uint32_t)(n[l] & 2) << 30));
    } else {
      const float v = (n[l] & 1) ? s[l] : c[l];
      y[l] = flip(v, (uint32_t)((n[l] ^ (n[l] >> 1)) & 1) << 31);
    }
  }
  y0 = y[0];
  y1 = y[1];
}

// finish over a group of P lanes, two at a time where finish2 applies
template <int K, bool F, int P, class T>
__device__ __forceinline__ void finish_group(const T (&a)[P], const T (&xr)[P], const int (&n)[P], T (&y)[P])
{
  if constexpr ((sincos_kind<K>::value || tancot_kind<K>::value) && std::is_same<T, float>::value && P % 2 == 0) {
#pragma unroll
    for (int l = 0; l < P; l += 2) finish2<K, F>(a[l], a[l + 1], xr[l], xr[l + 1], n[l], n[l + 1], y[l], y[l + 1]);
  } else {
#pragma unroll
    for (int l = 0; l < P; ++l) y[l] = finish<K, F>(a[l], xr[l], n[l]);
  }
}

// NT2's SIMD code over one pack of P lanes: y[l] = f(a[l]), one reduction
// method for the pack.  SIMD selects the packed-double conversion of the pi
// reduction (P > 1).
template <int K, bool F, int P, bool SIMD, class T>
__device__ __forceinline__ void pack_impl(const T (&a)[P], T (&y)[P])
{
  T x[P], xr[P];
  int n[P];
#pragma unroll
  for (int l = 0; l < P; ++l) x[l] = fabs(a[l]);
  if constexpr (pi_kind(K) || deg_kind(K)) {
#pragma unroll
    for (int l = 0; l < P; ++l) n[l] = reduce_unit<K>(x[l], xr[l], SIMD);
  } else {
    reduce_pack<P>(x, xr, n);
  }
  finish_group<K, F, P>(a, xr, n, y);
}
template <int K, bool F, int P, class T> __device__ __forceinline__ void pack(const T (&a)[P], T (&y)[P])
{
  pack_impl<K, F, P, (P > 1)>(a, y);
}

// ------------------------------------------------- inverse functions
// NT2's SIMD forms, element by element (no pack dependence):
// functions/simd/common/impl/invtrig/f_invtrig.hpp:31-110 and d_invtrig.hpp:29-139.
// seladd/ifadd/ifnotadd add a selected value (0 or c) unconditionally
// (boost/simd/boolean/functions/simd/common/{seladd,ifnotadd}.hpp); fms(a,b,c) = a*b - c.
struct tfi {
  static constexpr uint32_t pio2lo = 0xb33bbd2eu, pio4lo = 0xb2bbbd2eu, tan3pio8 = 0x401a827au,
                            tanpio8 = 0x3ed413cdu;
};
struct tdi {
  static constexpr uint64_t pio2lo = 0x3c91a62633145c07ull, pio4lo = 0x3c81a62633145c07ull,
                            tan3pio8 = 0x4003504f333f9de6ull, tanpio8 = 0x3fda827999fcef31ull,
                            sqrteps = 0x3e50000000000000ull;
};

template <bool F> __device__ __forceinline__ float asin(float a0)
{
  constexpr uint32_t P[5] = {0x3d2cb352u, 0x3cc617e3u, 0x3d3a3ec7u, 0x3d9980f6u, 0x3e2aaae4u};
  float x = fabsf(a0);
  const bool larger = x > 0.5f;
  float z = larger ? __fmul_rn(0.5f, __fsub_rn(1.0f, x)) : __fmul_rn(x, x);
  x = larger ? __fsqrt_rn(z) : x;
  float z1 = math::horner<F>(z, P);
  z1 = math::madd<F>(z1, __fmul_rn(z, x), x);
  z = larger ? __fsub_rn(fbits(tf::pio2), __fadd_rn(z1, z1)) : z1;
  return flip(z, sign_of(a0));
}
template <bool F> __device__ __forceinline__ float acos(float a0)
{
  float x = fabsf(a0);
  const bool larger = x > 0.5f;
  x = larger ? __fsqrt_rn(math::madd<F>(-0.5f, x, 0.5f)) : a0;
  x = asin<F>(x);
  x = __fadd_rn(x, larger ? x : 0.0f);
  x = (a0 < -0.5f) ? __fsub_rn(fbits(tf::pi), x) : x;
  return larger ? x : __fsub_rn(fbits(tf::pio2), x);
}
// atan(|a0|)
template <bool F> __device__ __forceinline__ float kernel_atan(float a0)
{
  constexpr uint32_t P[4] = {0x3da4f0d1u, 0xbe0e1b85u, 0x3e4c925fu, 0xbeaaaa2au};
  const float x = fabsf(a0);
  const bool flag1 = x < fbits(tfi::tan3pio8);
  const bool flag2 = flag1 && x >= fbits(tfi::tanpio8);
  float yy = flag1 ? 0.0f : fbits(tf::pio2);
  yy = flag2 ? fbits(tf::pio4) : yy;
  float xx = flag1 ? x : -__fdiv_rn(1.0f, x);
  xx = flag2 ? __fdiv_rn(__fsub_rn(x, 1.0f), __fadd_rn(x, 1.0f)) : xx;
  const float z = __fmul_rn(xx, xx);
  float z1 = math::madd<F>(xx, __fmul_rn(math::horner<F>(z, P), z), xx);
  z1 = __fadd_rn(z1, flag2 ? fbits(tfi::pio4lo) : 0.0f);
  z1 = __fadd_rn(z1, flag1 ? 0.0f : fbits(tfi::pio2lo));
  return __fadd_rn(yy, z1);
}
template <bool F> __device__ __forceinline__ float atan(float a0) { return flip(kernel_atan<F>(a0), sign_of(a0)); }
template <bool F> __device__ __forceinline__ double asin(double a0)
{
  constexpr uint64_t P1[5] = {0x3f684fc3988e9f08ull, 0xbfe2079259f9290full, 0x401bdff5baf33e6aull,
                              0xc03991aaac01ab68ull, 0x403c896240f3081dull};
  constexpr uint64_t Q1[5] = {0x3ff0000000000000ull, 0xc035f2a2b6bf5d8cull, 0x40626219af6a7f42ull,
                              0xc077fe08959063eeull, 0x40756709b0b644beull};
  constexpr uint64_t P2[6] = {0x3f716b9b0bd48ad3ull, 0xbfe34341333e5c16ull, 0x4015c74b178a2dd9ull,
                              0xc0304331de27907bull, 0x40339007da779259ull, 0xc020656c06ceafd5ull};
  constexpr uint64_t Q2[6] = {0x3ff0000000000000ull, 0xc02d7b590b5e0eabull, 0x40519fc025fe9054ull,
                              0xc06265bb6d3576d7ull, 0x4061705684ffbf9dull, 0xc04898220a3607acull};
  const double x = fabs(a0);
  double r;
  if (x < dbits(tdi::sqrteps)) {
    r = x;
  } else if (x > 0.625) {
    double zz1 = __dsub_rn(1.0, x);
    const double vp = __ddiv_rn(__dmul_rn(zz1, math::horner<F>(zz1, P1)), math::horner<F>(zz1, Q1));
    zz1 = __dsqrt_rn(__dadd_rn(zz1, zz1));
    double z = __dsub_rn(dbits(td::pio4), zz1);
    zz1 = F ? __fma_rn(zz1, vp, -dbits(tdi::pio2lo)) : __dsub_rn(__dmul_rn(zz1, vp), dbits(tdi::pio2lo));
    z = __dsub_rn(z, zz1);
    r = __dadd_rn(z, dbits(td::pio4));
  } else {
    const double zz2 = __dmul_rn(a0, a0);
    const double z = __ddiv_rn(__dmul_rn(zz2, math::horner<F>(zz2, P2)), math::horner<F>(zz2, Q2));
    r = math::madd<F>(x, z, x);
  }
  if (x > 1.0) return __longlong_as_double(0x7ff8000000000000ll);
  return flip(r, sign_of(a0));
}
template <bool F> __device__ __forceinline__ double acos(double a0)
{
  double x = fabs(a0);
  const bool larger = x > 0.5;
  x = larger ? __dsqrt_rn(math::madd<F>(-0.5, x, 0.5)) : a0;
  x = asin<F>(x);
  x = __dadd_rn(x, larger ? x : 0.0);
  x = (a0 < -0.5) ? __dsub_rn(dbits(td::pi), x) : x;
  return larger ? x : __dsub_rn(dbits(td::pio2), x);
}
// atan(|a0|)
template <bool F> __device__ __forceinline__ double kernel_atan(double a0)
{
  constexpr uint64_t P[5] = {0xbfec007fa1f72594ull, 0xc03028545b6b807aull, 0xc052c08c36880273ull,
                             0xc05eb8bf2d05ba25ull, 0xc0503669fd28ec8eull};
  constexpr uint64_t Q[6] = {0x3ff0000000000000ull, 0x4038dbc45b14603cull, 0x4064a0dd43b8fa25ull,
                             0x407b0e18d2e2be3bull, 0x407e563f13b049eaull, 0x4068519efbbd62ecull};
  const double x = fabs(a0);
  const bool flag1 = x < dbits(tdi::tan3pio8);
  const bool flag2 = flag1 && x >= dbits(tdi::tanpio8);
  double yy = flag1 ? 0.0 : dbits(td::pio2);
  yy = flag2 ? dbits(td::pio4) : yy;
  double xx = flag1 ? x : -__ddiv_rn(1.0, x);
  xx = flag2 ? __ddiv_rn(__dsub_rn(x, 1.0), __dadd_rn(x, 1.0)) : xx;
  double z = __dmul_rn(xx, xx);
  z = __ddiv_rn(__dmul_rn(z, math::horner<F>(z, P)), math::horner<F>(z, Q));
  z = math::madd<F>(xx, z, xx);
  z = __dadd_rn(z, flag2 ? dbits(tdi::pio4lo) : 0.0);
  z = __dadd_rn(z, flag1 ? 0.0 : dbits(tdi::pio2lo));
  return __dadd_rn(yy, z);
}
template <bool F> __device__ __forceinline__ double atan(double a0) { return flip(kernel_atan<F>(a0), sign_of(a0)); }

// atan2(a0, a1), NT2's SIMD form (functions/simd/common/atan2.hpp:31-52): both
// infinite -> +-1 each; kernel_atan(a0/a1); Pi minus it unless a1 > 0; the sign
// of a0 (negatenz: -0 counts as negative); a0 == 0 -> (a1 < 0 ? Pi : 0); NaN if
// either argument is NaN.
template <bool F, class T> __device__ __forceinline__ T atan2(T a0, T a1)
{
  const T pi = sizeof(T) == 4 ? (T)fbits(tf::pi) : (T)dbits(td::pi);
  if (isinf(a0) && isinf(a1)) {
    a0 = copysign(T(1), a0);
    a1 = copysign(T(1), a1);
  }
  T z = kernel_atan<F>(math::div(a0, a1));
  z = (a1 > T(0)) ? z : math::sub(pi, z);
  z = flip(z, sign_of(a0));
  z = (a0 == T(0)) ? ((a1 < T(0)) ? pi : T(0)) : z;
  return (isnan(a0) || isnan(a1)) ? (T)NAN : z;
}

// One element, NT2's scalar code (a pack of one).
template <int K, bool F, class T> __device__ __forceinline__ T one(T a)
{
  T in[1] = {a}, out[1];
  pack_impl<K, F, 1, false>(in, out);
  return out[0];
}

// NT2's scalar code on the P elements of a thread's group, each reduced on its
// own.  Levels 0-2 (|x| <= 20 pi) are computed without branches: the cephes
// and straight reductions are both evaluated and the element's level picks
// between them and x itself, so a warp whose elements mix these levels runs
// one path.  Larger levels branch per element.
template <class T> __device__ __forceinline__ int reduce_low(int lv, T x, T& xr)
{
  T xs, xc;
  straight(x, xs);
  const int nc = cephes(x, xc);
  xr = lv == 0 ? x : (lv == 1 ? xs : xc);
  return lv == 0 ? 0 : (lv == 1 ? 1 : nc);
}
// reduce_low for two float elements whose levels are both at most 2, on the
// packed instructions: the straight and cephes chains are the scalar ones
// lane by lane (each product that feeds a subtraction formed by x2::mul_r);
// cephes' quotient rint(x*2/pi) is at most 40 here, so it is (v + 1.5*2^23)
// - 1.5*2^23, and its low bits are those of the sum.
__device__ __forceinline__ void reduce_low2(int lv0, int lv1, float x0, float x1, float& xr0, float& xr1, int& n0,
                                            int& n1)
{
  using x2::splat;
  const float2 x = make_float2(x0, x1);
  float2 xs = x2::sub(x, splat(fbits(tf::pio2_1)));
  xs = x2::sub(xs, splat(fbits(tf::pio2_2)));
  xs = x2::sub(xs, splat(fbits(tf::pio2_3)));
  const float2 t = x2::add(x2::mul_r(x, splat(fbits(tf::twoopi))), splat(x2::kRound));
  const float2 xi = x2::sub(t, splat(x2::kRound));
  float2 xc = x2::sub(x, x2::mul_r(xi, splat(fbits(tf::pio2_1))));
  xc = x2::sub(xc, x2::mul_r(xi, splat(fbits(tf::pio2_2))));
  xc = x2::sub(xc, x2::mul_r(xi, splat(fbits(tf::pio2_3))));
  const int nc0 = (int)(__float_as_uint(t.x) & 3u), nc1 = (int)(__float_as_uint(t.y) & 3u);
  xr0 = lv0 == 0 ? x0 : (lv0 == 1 ? xs.x : xc.x);
  xr1 = lv1 == 0 ? x1 : (lv1 == 1 ? xs.y : xc.y);
  n0 = lv0 == 0 ? 0 : (lv0 == 1 ? 1 : nc0);
  n1 = lv1 == 0 ? 0 : (lv1 == 1 ? 1 : nc1);
}
template <int K, bool F, int P, class T> __device__ __forceinline__ void scalar_group(const T (&a)[P], T (&y)[P])
{
  if constexpr (pi_kind(K) || deg_kind(K)) {
    pack_impl<K, F, P, false>(a, y);
  } else if constexpr (std::is_same<T, float>::value && P % 2 == 0) {
    T xr[P];
    int n[P];
#pragma unroll
    for (int l = 0; l < P; l += 2) {
      const T xa = fabs(a[l]), xb = fabs(a[l + 1]);
      const int la = level(xa), lb = level(xb);
      if (la <= 2 && lb <= 2) {
        reduce_low2(la, lb, xa, xb, xr[l], xr[l + 1], n[l], n[l + 1]);
      } else {
        T x1[1] = {xa}, r1[1];
        int n1[1];
        if (la <= 2) n1[0] = reduce_low(la, xa, r1[0]);
        else reduce_at<1>(la, x1, r1, n1);
        xr[l] = r1[0];
        n[l] = n1[0];
        x1[0] = xb;
        if (lb <= 2) n1[0] = reduce_low(lb, xb, r1[0]);
        else reduce_at<1>(lb, x1, r1, n1);
        xr[l + 1] = r1[0];
        n[l + 1] = n1[0];
      }
    }
    finish_group<K, F, P>(a, xr, n, y);
  } else {
    T xr[P];
    int n[P];
#pragma unroll
    for (int l = 0; l < P; ++l) {
      T x1[1] = {fabs(a[l])}, r1[1];
      int n1[1];
      const int lv = level(x1[0]);
      if (lv <= 2) {
        n1[0] = reduce_low(lv, x1[0], r1[0]);
      } else {
        reduce_at<1>(lv, x1, r1, n1);
      }
      xr[l] = r1[0];
      n[l] = n1[0];
    }
    finish_group<K, F, P>(a, xr, n, y);
  }
}

// ----------------------------------------------------------- compositions
// The steps NT2's composed trigonometric functors add around sin, cos, sinpi,
// cospi, asin, acos, atan (modules/core/trigonometric/include/nt2/trigonometric/
// functions/generic/{indeg,inrad,asinpi,cscd,asec,cscpi,secpi}.hpp), constants as
// bit patterns of their BOOST_SIMD_CONSTANT_REGISTER lines.
// indeg(x) = x*Radindeg - x*Radindegr (the second constant is the rounding residual of 180/pi)
__device__ __forceinline__ float indeg(float a)
{ return math::sub(math::mul(a, __uint_as_float(0x42652ee1u)), math::mul(a, __uint_as_float(0xb53387c1u))); }
__device__ __forceinline__ double indeg(double a)
{
  return math::sub(math::mul(a, math::dbits(0x404ca5dc1a63c1f8ull)), math::mul(a, math::dbits(0xbce1e7ab456405f8ull)));
}
__device__ __forceinline__ float inrad(float a) { return math::mul(a, __uint_as_float(0x3c8efa35u)); }
__device__ __forceinline__ double inrad(double a) { return math::mul(a, math::dbits(0x3f91df46a2529d39ull)); }
__device__ __forceinline__ float invpi_mul(float a) { return math::mul(__uint_as_float(0x3ea2f983u), a); }
__device__ __forceinline__ double invpi_mul(double a) { return math::mul(math::dbits(0x3fd45f306dc9c883ull), a); }
__device__ __forceinline__ float oneo_180_mul(float a) { return math::mul(__uint_as_float(0x3bb60b61u), a); }
__device__ __forceinline__ double oneo_180_mul(double a) { return math::mul(math::dbits(0x3f76c16c16c16c17ull), a); }
__device__ __forceinline__ float pio2_minus(float a) { return math::sub(__uint_as_float(0x3fc90fdbu), a); }
__device__ __forceinline__ double pio2_minus(double a) { return math::sub(math::dbits(0x3ff921fb54442d18ull), a); }
// cscpi: NaN where x is a nonzero integer; secpi: NaN where 2x is odd (is_odd(y) =
// is_flint((y - 1) / 2)); elsewhere the reciprocal v computed beside it
template <class T> __device__ __forceinline__ T cscpi_nan(T x, T v)
{ return (math::is_flint(x) && x != T(0)) ? T(NAN) : v; }
template <class T> __device__ __forceinline__ T secpi_nan(T x, T v)
{ return math::is_flint(math::mul(math::sub(math::mul(x, T(2)), T(1)), T(0.5))) ? T(NAN) : v; }

// ------------------------------------------------------------ fast forms
// fast_sin ... fast_cotd (generic/fast_<name>.hpp: trig_base with the clipped_pio4_
// mode, NT2's "fast" style, functions/simd/common/impl/trigo/trig_base.hpp:67-135,
// 143-149): no reduction; x = (|x| > max_range ? NaN : x) * scale, (max_range,
// scale) = (pi/4, 1) radians, (1/4, pi) half turns, (45, Pio_180) degrees; then the
// kind's polynomial.  K: 0 sin, 1 cos, 2 tan, 3 cot; U: 0 radian, 1 pi, 2 degree.
template <int K, int U, bool F, class T> __device__ __forceinline__ T fast(T a0)
{
  constexpr bool S = sizeof(T) == 4;
  const T range = U == 0 ? (S ? (T)fbits(0x3f490fdbu) : (T)dbits(0x3fe921fb54442d18ull)) : (U == 1 ? T(0.25) : T(45));
  T x = fabs(a0) > range ? T(NAN) : a0;
  if constexpr (U == 1) x = math::mul(x, S ? (T)fbits(tf::pi) : (T)dbits(td::pi));
  if constexpr (U == 2) x = math::mul(x, S ? (T)fbits(0x3c8efa35u) : (T)dbits(0x3f91df46a2529d3aull));
  if constexpr (K == 0) return sin_eval<F>(math::mul(x, x), x);
  else if constexpr (K == 1) return cos_eval<F>(math::mul(x, x));
  else if constexpr (K == 2) return tan_eval<F>(x);
  else return math::div(T(1), tan_eval<F>(x));
}
// proper_tanpi (simd/common/proper_tanpi.hpp:33-43): fast_tanpi of |x| (|x| <= 1/4) or of
// 1/2 - |x| and its reciprocal, the sign of x, NaN unless |x| <= 1/2
template <bool F, class T> __device__ __forceinline__ T proper_tanpi(T a0)
{
  const T ax = fabs(a0);
  const bool test = ax <= T(0.25);
  T t = fast<2, 1, F>(test ? ax : math::sub(T(0.5), ax));
  t = a0 < T(0) ? -t : t;
  return !(ax <= T(0.5)) ? T(NAN) : (test ? t : math::div(T(1), t));
}
// sinc / sincpi final steps (simd/common/sinc.hpp:33-45, sincpi.hpp:33-45): 1 where
// |x| < Eps, 0 where x is infinite, else the quotient r computed beside it
template <class T> __device__ __forceinline__ T sinc_fix(T x, T r)
{
  const T eps = sizeof(T) == 4 ? (T)fbits(0x34000000u) : (T)dbits(0x3cb0000000000000ull);
  r = fabs(x) < eps ? T(1) : r;
  return isinf(x) ? T(0) : r;
}
// nbd_atan2 (simd/common/nbd_atan2.hpp:35-42): atan2 without its infinity and NaN cases
template <bool F, class T> __device__ __forceinline__ T nbd_atan2(T a0, T a1)
{
  const T pi = sizeof(T) == 4 ? (T)fbits(tf::pi) : (T)dbits(td::pi);
  T z = kernel_atan<F>(math::div(a0, a1));
  z = (a1 > T(0)) ? z : math::sub(pi, z);
  z = flip(z, sign_of(a0));
  return (a0 == T(0)) ? ((a1 < T(0)) ? pi : T(0)) : z;
}

}  // namespace trig
}  // namespace nt2cuda
