// nt2cuda/math.cuh -- NT2's elementwise math functors on sm_103a.
//
// Each functor follows the NT2 algorithm that the SIMD transform body runs
// (file:line cited per function, paths relative to the NT2 source tree).
// NT2's generic fma/fnms are `a*b+c` rounded twice
// (modules/boost/simd/base/include/boost/simd/arithmetic/functions/generic/fma.hpp:32),
// so the default here (Fused = false) spells every multiply and add with the
// _rn intrinsics: nvcc never contracts them, whatever flags the including
// translation unit uses, and the results are bit-identical to NT2 evaluated
// without contraction.  Fused = true turns each NT2 fma/fnms/horner step into
// one hardware FMA, which is what NT2 compiled with FMA contraction computes;
// its ULP distance to the unfused form is measured by the parity tests.
// Division and square root are always the IEEE-rounded forms, as in NT2.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nt2cuda {
namespace math {

// ------------------------------------------------------------ primitives
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }

// NT2 fma(a,b,c) = a*b+c ; fnms(a,b,c) = c-a*b
template <bool F> __device__ __forceinline__ float madd(float a, float b, float c)
{ return F ? __fmaf_rn(a, b, c) : __fadd_rn(__fmul_rn(a, b), c); }
template <bool F> __device__ __forceinline__ float nmsub(float a, float b, float c)
{ return F ? __fmaf_rn(-a, b, c) : __fsub_rn(c, __fmul_rn(a, b)); }
template <bool F> __device__ __forceinline__ double madd(double a, double b, double c)
{ return F ? __fma_rn(a, b, c) : __dadd_rn(__dmul_rn(a, b), c); }
template <bool F> __device__ __forceinline__ double nmsub(double a, double b, double c)
{ return F ? __fma_rn(-a, b, c) : __dsub_rn(c, __dmul_rn(a, b)); }

__device__ __forceinline__ float fbits(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ double dbits(uint64_t u) { return __longlong_as_double((long long)u); }

// Static Horner, coefficients (bit patterns) in decreasing powers:
// modules/core/polynomials/include/nt2/polynomials/functions/scalar/impl/horner.hpp:26-45
template <bool F, int N>
__device__ __forceinline__ float horner(float x, const uint32_t (&c)[N])
{
  float acc = fbits(c[0]);
#pragma unroll
  for (int i = 1; i < N; ++i) acc = madd<F>(x, acc, fbits(c[i]));
  return acc;
}
template <bool F, int N>
__device__ __forceinline__ double horner(double x, const uint64_t (&c)[N])
{
  double acc = dbits(c[0]);
#pragma unroll
  for (int i = 1; i < N; ++i) acc = madd<F>(x, acc, dbits(c[i]));
  return acc;
}

// --------------------------------------------------------------- constants
// Bit patterns from each constant's BOOST_SIMD_CONSTANT_REGISTER line.
struct cf {
  static constexpr uint32_t maxlog = 0x42b0c0a5u, minlog = 0xc2b0c0a5u, invlog_2 = 0x3fb8aa3bu,
                            log_2hi = 0x3f318000u, log_2lo = 0xb95e8083u, sqrt_2o_2 = 0x3f3504f3u,
                            twothird = 0x3f2aaaabu, invsqrt_2pi = 0x3ecc422au,
                            smallestposval = 0x00800000u, twotonmb = 0x4b000000u,
                            mlogtwo2nmb = 0xc17f1402u;
};
struct cd {
  static constexpr uint64_t maxlog = 0x40862e42fefa39efull, minlog = 0xc086232bdd7abcd2ull,
                            invlog_2 = 0x3ff71547652b82feull, log_2hi = 0x3fe62e42fee00000ull,
                            log_2lo = 0x3dea39ef35793c76ull, sqrt_2o_2 = 0x3fe6a09e667f3bcdull;
};

// ---------------------------------------------------------------- float exp
// reduce/approx: modules/core/exponential/include/nt2/exponential/functions/scalar/impl/expo/f_expo_reduction.hpp:62-85
// selections:    .../exponential/functions/simd/common/impl/expo/expo_base.hpp:48-62
// scale by 2^k:  .../exponential/functions/scalar/impl/expo/expo_scale.hpp:26-35
template <bool F = false>
__device__ __forceinline__ float exp(float a0)
{
  constexpr uint32_t P[5] = {0x3ab778cfu, 0x3c098d8bu, 0x3d2aa957u, 0x3e2aa9a5u, 0x3f000000u};
  float k = rintf(mul(fbits(cf::invlog_2), a0));
  float x = nmsub<F>(k, fbits(cf::log_2hi), a0);
  x = nmsub<F>(k, fbits(cf::log_2lo), x);
  float y = horner<F>(x, P);
  float c = add(madd<F>(y, mul(x, x), x), 1.0f);
  unsigned ik = (unsigned)((int)k + 127);              // k in [-127,127] on the kept lanes
  float r = mul(c, __uint_as_float(ik << 23));
  r = (a0 <= fbits(cf::minlog)) ? 0.0f : r;
  r = (a0 >= fbits(cf::maxlog)) ? __int_as_float(0x7f800000) : r;
  return (a0 != a0) ? a0 : r;
}

// ---------------------------------------------------------------- float log
// modules/core/exponential/include/nt2/exponential/functions/simd/common/impl/logs/f_log.hpp:101-124, finalize :173-186
// kernel: .../exponential/functions/scalar/impl/logs/f_kernel.hpp:43-73
template <bool F = false>
__device__ __forceinline__ float log(float a0)
{
  constexpr uint32_t P[8] = {0xbda5dff0u, 0x3e0229f9u, 0xbe04d6b7u, 0x3e116e80u,
                             0xbe2a6aa0u, 0x3e4cd0a3u, 0xbe800064u, 0x3eaaaaa9u};
  float z = a0, t = 0.0f;
  if (fabsf(z) < fbits(cf::smallestposval)) { z = mul(z, fbits(cf::twotonmb)); t = fbits(cf::mlogtwo2nmb); }
  uint32_t u = __float_as_uint(z);
  int e = (int)((u & 0x7f800000u) >> 23) - 126;
  float x = __uint_as_float((u & ~0x7f800000u) | 0x3f000000u);   // fast_frexp
  bool lt = x < fbits(cf::sqrt_2o_2);
  float fe = lt ? add((float)e, -1.0f) : (float)e;
  x = sub(lt ? add(x, x) : x, 1.0f);
  float x2 = mul(x, x);
  float y = mul(mul(horner<F>(x, P), x), x2);
  y = madd<F>(fe, fbits(cf::log_2lo), y);
  y = madd<F>(-0.5f, x2, y);
  float r = madd<F>(fbits(cf::log_2hi), fe, add(add(x, y), t));
  r = (a0 < 0.0f || a0 != a0) ? __int_as_float(0x7fffffff) : r;
  r = (a0 == __int_as_float(0x7f800000)) ? a0 : r;
  return (a0 == 0.0f) ? __int_as_float(0xff800000) : r;
}

// ----------------------------------------------- exp2, exp10, log2, log10
// The exp and log skeletons with NT2's other reductions and recombinations:
// exp2/exp10 float: modules/core/exponential/include/nt2/exponential/functions/scalar/impl/expo/f_expo_reduction.hpp:88-143,
// log2/log10 float: .../functions/simd/common/impl/logs/f_log.hpp:126-170 (constants: exponential/constants/*.hpp).
struct cf2 {
  static constexpr uint32_t maxlog2 = 0x42fe0000u, minlog2 = 0xc2fe0000u, maxlog10 = 0x4218ec59u,
                            minlog10 = 0xc2179999u, invlog10_2 = 0x40549a78u, log10_2hi = 0x3e9a0000u,
                            log10_2lo = 0x39826a14u, log_2 = 0x3f317218u, log2_em1 = 0x3ee2a8edu,
                            log10_elo = 0x3a37b152u, log10_ehi = 0x3ede0000u, mlog2two2nmb = 0xc1b80000u,
                            mlog10two2nmb = 0xc0dd8edeu;
};

// expo_base selections (simd/common/impl/expo/expo_base.hpp:48-62) and the
// exponent-bit scale by 2^k (scalar/impl/expo/expo_scale.hpp:26-35)
__device__ __forceinline__ float expo_select(float a0, float c, float k, float minl, float maxl)
{
  unsigned ik = (unsigned)((int)k + 127);
  float r = mul(c, __uint_as_float(ik << 23));
  r = (a0 <= minl) ? 0.0f : r;
  r = (a0 >= maxl) ? __int_as_float(0x7f800000) : r;
  return (a0 != a0) ? a0 : r;
}

template <bool F = false>
__device__ __forceinline__ float exp2(float a0)
{
  constexpr uint32_t P[5] = {0x3922c8c4u, 0x3ab01218u, 0x3c1d9422u, 0x3d6356ebu, 0x3e75fdf1u};
  float k = rintf(a0);
  float x = sub(a0, k);
  float y = horner<F>(x, P);
  float c = add(madd<F>(y, mul(x, x), mul(x, fbits(cf2::log_2))), 1.0f);   // inc(fma(y, sqr(x), x*Log_2))
  return expo_select(a0, c, k, fbits(cf2::minlog2), fbits(cf2::maxlog2));
}

template <bool F = false>
__device__ __forceinline__ float exp10(float a0)
{
  constexpr uint32_t P[6] = {0x3e54dff1u, 0x3f0aacefu, 0x3f95eb4cu, 0x400237dau, 0x4029a926u, 0x40135d8eu};
  float k = rintf(mul(fbits(cf2::invlog10_2), a0));
  float x = nmsub<F>(k, fbits(cf2::log10_2hi), a0);
  x = nmsub<F>(k, fbits(cf2::log10_2lo), x);
  float c = madd<F>(horner<F>(x, P), x, 1.0f);                               // inc(horner(x)*x)
  return expo_select(a0, c, k, fbits(cf2::minlog10), fbits(cf2::maxlog10));
}

// the float log kernel (scalar/impl/logs/f_kernel.hpp:43-73) after f_log.hpp's denormal rescale
struct logparts { float fe, x, x2, y, t; };
template <bool F>
__device__ __forceinline__ logparts log_kernel(float a0, float mtwo2nmb)
{
  constexpr uint32_t P[8] = {0xbda5dff0u, 0x3e0229f9u, 0xbe04d6b7u, 0x3e116e80u,
                             0xbe2a6aa0u, 0x3e4cd0a3u, 0xbe800064u, 0x3eaaaaa9u};
  logparts p;
  float z = a0;
  p.t = 0.0f;
  if (fabsf(z) < fbits(cf::smallestposval)) { z = mul(z, fbits(cf::twotonmb)); p.t = mtwo2nmb; }
  uint32_t u = __float_as_uint(z);
  int e = (int)((u & 0x7f800000u) >> 23) - 126;
  float x = __uint_as_float((u & ~0x7f800000u) | 0x3f000000u);   // fast_frexp
  bool lt = x < fbits(cf::sqrt_2o_2);
  p.fe = lt ? add((float)e, -1.0f) : (float)e;
  p.x = sub(lt ? add(x, x) : x, 1.0f);
  p.x2 = mul(p.x, p.x);
  p.y = mul(mul(horner<F>(p.x, P), p.x), p.x2);
  return p;
}

// f_log.hpp finalize (:173-186)
__device__ __forceinline__ float log_finalize(float a0, float r)
{
  r = (a0 < 0.0f || a0 != a0) ? __int_as_float(0x7fffffff) : r;
  r = (a0 == __int_as_float(0x7f800000)) ? a0 : r;
  return (a0 == 0.0f) ? __int_as_float(0xff800000) : r;
}

template <bool F = false>
__device__ __forceinline__ float log2(float a0)
{
  logparts p = log_kernel<F>(a0, fbits(cf2::mlog2two2nmb));
  float y = madd<F>(-0.5f, p.x2, p.y);
  float z = madd<F>(p.x, fbits(cf2::log2_em1), mul(y, fbits(cf2::log2_em1)));
  return log_finalize(a0, add(add(add(add(z, y), p.x), p.fe), p.t));
}

template <bool F = false>
__device__ __forceinline__ float log10(float a0)
{
  logparts p = log_kernel<F>(a0, fbits(cf2::mlog10two2nmb));
  float y = madd<F>(-0.5f, p.x2, p.y);                       // amul(y, Mhalf, x2)
  float z = mul(add(p.x, y), fbits(cf2::log10_elo));
  z = madd<F>(y, fbits(cf2::log10_ehi), z);                  // amul(z, y, Log10_ehi)
  z = madd<F>(p.x, fbits(cf2::log10_ehi), z);
  z = madd<F>(p.fe, fbits(cf2::log10_2hi), z);
  return log_finalize(a0, madd<F>(p.fe, fbits(cf2::log10_2lo), add(z, p.t)));
}

// ---------------------------------------------------------- expm1, log1p
// expm1: modules/core/exponential/include/nt2/exponential/functions/details/expm1_kernel.hpp:24-80,
// selections simd/common/expm1.hpp:35-41, fast_ldexp by exponent bits;
// log1p: .../functions/simd/common/log1p.hpp:29-38.
template <bool F = false>
__device__ __forceinline__ float expm1(float a0)
{
  constexpr uint32_t P[3] = {0x3acf6db4u, 0xbd08887fu, 0x3f800000u};
  float k = rintf(mul(fbits(cf::invlog_2), a0));
  float x = nmsub<F>(k, fbits(cf::log_2hi), a0);
  x = nmsub<F>(k, fbits(cf::log_2lo), x);
  float hx = mul(x, 0.5f);
  float hxs = mul(x, hx);
  float r1 = horner<F>(hxs, P);
  float t = nmsub<F>(r1, hx, 3.0f);                          // fnms(r1, hx, Three)
  float e = mul(hxs, div(sub(r1, t), nmsub<F>(x, t, 6.0f)));
  e = F ? __fmaf_rn(x, e, -hxs) : sub(mul(x, e), hxs);      // fms(x, e, hxs)
  int ik = (int)k;
  float two2mk = __uint_as_float((unsigned)(127 - ik) << 23);
  float y = sub(sub(1.0f, two2mk), sub(e, x));
  float r = mul(y, __uint_as_float((unsigned)(ik + 127) << 23));
  r = (a0 > fbits(cf::maxlog)) ? __int_as_float(0x7f800000) : r;
  return (a0 < __uint_as_float(0xc17f1402u)) ? -1.0f : r;    // Logeps
}

template <bool F = false>
__device__ __forceinline__ float log1p(float a0)
{
  float u = add(1.0f, a0);
  float r = log<F>(u);
  r = (u != 0.0f) ? add(r, div(sub(a0, sub(u, 1.0f)), u)) : r;
  return (u == __int_as_float(0x7f800000)) ? u : r;
}

// --------------------------------------------------------------- float erfc
// modules/core/euler/include/nt2/euler/functions/simd/common/erfc.hpp:92-121
// kernels: modules/core/euler/include/nt2/euler/functions/details/erf_kernel.hpp:48-85
// erfc_abs(x) is the |a0| part, shared by erfc(a) and erfc(-a):
// erfc(a) = a < 0 ? 2 - erfc_abs(|a|) : erfc_abs(|a|).
// The two regions of NT2's float erfc, given x = |a| and z = x/(1+x).
template <bool F = false>
__device__ __forceinline__ float erfc_small(float z)
{
  constexpr uint32_t P3[9] = {0x41aa8e55u, 0x401b5680u, 0xc010d956u, 0x3f2cff3bu,
                              0xc016c985u, 0xbffc9284u, 0xbfa11698u, 0xbe036d7eu, 0x3f7ffffeu};
  return mul(sub(1.0f, z), horner<F>(z, P3));
}
template <bool F = false>
__device__ __forceinline__ float erfc_large(float x, float z)
{
  constexpr uint32_t P2[11] = {0xc0283611u, 0x40d67e3bu, 0xc0cd1a85u, 0x4050b063u,
                               0xbfaea865u, 0x3e2006f0u, 0x3e1175c7u, 0x3ec4ca6eu,
                               0x3e243828u, 0xbf918a62u, 0x3f0a0e8bu};
  return mul(exp<F>(-mul(x, x)), horner<F>(sub(z, 0.4f), P2));
}
__device__ __forceinline__ bool erfc_is_small(float x) { return x < fbits(cf::twothird); }
__device__ __forceinline__ float erfc_finish(float x, float r1)
{
  return (x == __int_as_float(0x7f800000)) ? 0.0f : r1;
}

template <bool F = false>
__device__ __forceinline__ float erfc_abs(float x)
{
  float z = div(x, add(1.0f, x));
  float r1 = erfc_is_small(x) ? erfc_small<F>(z) : erfc_large<F>(x, z);
  return erfc_finish(x, r1);
}

template <bool F = false>
__device__ __forceinline__ float erfc(float a0)
{
  float r1 = erfc_abs<F>(fabsf(a0));
  return (a0 < 0.0f) ? sub(2.0f, r1) : r1;
}

// normcdf(x) = 0.5*erfc(-sqrt(2)/2 * x):
// modules/core/statistics/include/nt2/statistics/functions/generic/normcdf.hpp:28-34
template <bool F = false>
__device__ __forceinline__ float normcdf(float a0)
{
  return mul(0.5f, erfc<F>(mul(-fbits(cf::sqrt_2o_2), a0)));
}

// normcdf(x) and normcdf(-x) from one erfc core.  normcdf(-x) evaluates
// erfc(+c*x) = erfc(-(-c*x)), and erfc only looks at the sign and |arg|,
// so both results are bit-identical to two separate normcdf calls.
template <bool F = false>
__device__ __forceinline__ void normcdf_pair(float a0, float& pos, float& neg)
{
  float y = mul(-fbits(cf::sqrt_2o_2), a0);
  float r1 = erfc_abs<F>(fabsf(y));
  float two_m = sub(2.0f, r1);
  pos = mul(0.5f, (y < 0.0f) ? two_m : r1);
  neg = mul(0.5f, (-y < 0.0f) ? two_m : r1);
}

// fastnormcdf (Abramowitz-Stegun 26.2.17):
// modules/core/statistics/include/nt2/statistics/functions/generic/fastnormcdf.hpp:33-53
template <bool F = false>
__device__ __forceinline__ float fastnormcdf(float a0)
{
  constexpr uint32_t P[5] = {0x3faa466fu, 0xbfe91eeau, 0x3fe40778u, 0xbeb68f87u, 0x3ea385fau};
  float l = fabsf(a0);
  float k = div(1.0f, madd<F>(0.2316419f, l, 1.0f));
  float w = horner<F>(k, P);
  w = mul(w, mul(mul(k, fbits(cf::invsqrt_2pi)), exp<F>(mul(-mul(l, l), 0.5f))));
  return (a0 > 0.0f) ? sub(1.0f, w) : w;
}

// fastnormcdf(x) and fastnormcdf(-x): w depends on |x| only.
template <bool F = false>
__device__ __forceinline__ void fastnormcdf_pair(float a0, float& pos, float& neg)
{
  constexpr uint32_t P[5] = {0x3faa466fu, 0xbfe91eeau, 0x3fe40778u, 0xbeb68f87u, 0x3ea385fau};
  float l = fabsf(a0);
  float k = div(1.0f, madd<F>(0.2316419f, l, 1.0f));
  float w = horner<F>(k, P);
  w = mul(w, mul(mul(k, fbits(cf::invsqrt_2pi)), exp<F>(mul(-mul(l, l), 0.5f))));
  float om = sub(1.0f, w);
  pos = (a0 > 0.0f) ? om : w;
  neg = (-a0 > 0.0f) ? om : w;
}

// --------------------------------------------------------------- double exp
// modules/core/exponential/include/nt2/exponential/functions/scalar/impl/expo/d_expo_reduction.hpp:57-82
// selections: .../exponential/functions/simd/common/impl/expo/expo_base.hpp:31-45
template <bool F = false>
__device__ __forceinline__ double exp(double a0)
{
  constexpr uint64_t P[5] = {0x3e66376972bea4d0ull, 0xbebbbd41c5d26bf1ull, 0x3f11566aaf25de2cull,
                             0xbf66c16c16bebd93ull, 0x3fc555555555553eull};
  double k = rint(mul(dbits(cd::invlog_2), a0));
  double hi = nmsub<F>(k, dbits(cd::log_2hi), a0);
  double lo = mul(k, dbits(cd::log_2lo));
  double x = sub(hi, lo);
  double t = mul(x, x);
  double c = nmsub<F>(t, horner<F>(t, P), x);
  c = sub(1.0, sub(sub(lo, div(mul(x, c), sub(2.0, c))), hi));
  unsigned long long ik = (unsigned long long)((long long)k + 1023);
  double r = mul(c, __longlong_as_double((long long)(ik << 52)));
  r = (a0 <= dbits(cd::minlog)) ? 0.0 : r;
  r = (a0 >= dbits(cd::maxlog)) ? __longlong_as_double(0x7ff0000000000000ll) : r;
  return (a0 != a0) ? a0 : r;
}

// --------------------------------------------------------------- double log
// modules/core/exponential/include/nt2/exponential/functions/simd/common/impl/logs/d_log.hpp:57-98, finalize :124-137
template <bool F = false>
__device__ __forceinline__ double log(double a0)
{
  constexpr uint64_t T1[3] = {0x3fc39a09d078c69full, 0x3fcc71c51d8e78afull, 0x3fd999999997fa04ull};
  constexpr uint64_t T2[4] = {0x3fc2f112df3e5244ull, 0x3fc7466496cb03deull, 0x3fd2492494229359ull,
                              0x3fe5555555555593ull};
  unsigned long long u = (unsigned long long)__double_as_longlong(a0);
  long long k = (long long)((u & 0x7ff0000000000000ull) >> 52) - 1022;
  double x = __longlong_as_double((long long)((u & ~0x7ff0000000000000ull) | 0x3fe0000000000000ull));
  bool lt = dbits(cd::sqrt_2o_2) > x;
  k = k + (lt ? -1 : 0);
  double f = sub(add(x, lt ? x : 0.0), 1.0);
  double dk = (double)k;
  double s = div(f, add(2.0, f));
  double z = mul(s, s);
  double w = mul(z, z);
  double t1 = mul(w, horner<F>(w, T1));
  double t2 = mul(z, horner<F>(w, T2));
  double R = add(t2, t1);
  double hfsq = mul(0.5, mul(f, f));
  double y = sub(mul(dk, dbits(cd::log_2hi)),
                 sub(sub(hfsq, madd<F>(s, add(hfsq, R), mul(dk, dbits(cd::log_2lo)))), f));
  y = (a0 < 0.0 || a0 != a0) ? __longlong_as_double(0x7fffffffffffffffll) : y;
  y = (a0 == __longlong_as_double(0x7ff0000000000000ll)) ? a0 : y;
  return (a0 == 0.0) ? __longlong_as_double((long long)0xfff0000000000000ull) : y;
}

// ------------------------------------ double exp2, exp10, log2, log10
// exp2/exp10: .../scalar/impl/expo/d_expo_reduction.hpp:85-160 with expo_base.hpp:26-45;
// log2/log10: .../simd/common/impl/logs/d_log.hpp:99-121.
struct cd2 {
  static constexpr uint64_t maxlog2 = 0x408ff80000000000ull, minlog2 = 0xc08ff00000000000ull,
                            maxlog10 = 0x40734413509f79feull, minlog10 = 0xc0734413509f79feull,
                            invlog10_2 = 0x400a934f0979a372ull, log10_2hi = 0x3fd3440000000000ull,
                            log10_2lo = 0x3ed3509f79fef312ull, log_2 = 0x3fe62e42fefa39efull,
                            invlog_10 = 0x3fdbcb7b1526e50dull, log_2olog_10 = 0x3fd34413509f79ffull;
};

__device__ __forceinline__ double expo_select(double a0, double c, double k, double minl, double maxl)
{
  unsigned long long ik = (unsigned long long)((long long)k + 1023);
  double r = mul(c, __longlong_as_double((long long)(ik << 52)));
  r = (a0 <= minl) ? 0.0 : r;
  r = (a0 >= maxl) ? __longlong_as_double(0x7ff0000000000000ll) : r;
  return (a0 != a0) ? a0 : r;
}

template <bool F = false>
__device__ __forceinline__ double exp2(double a0)
{
  constexpr uint64_t P[5] = {0x3e66376972bea4d0ull, 0xbebbbd41c5d26bf1ull, 0x3f11566aaf25de2cull,
                             0xbf66c16c16bebd93ull, 0x3fc555555555553eull};
  double k = rint(a0);
  double x = mul(sub(a0, k), dbits(cd2::log_2));
  double t = mul(x, x);
  double c = nmsub<F>(t, horner<F>(t, P), x);
  c = sub(1.0, sub(div(-mul(x, c), sub(2.0, c)), x));       // oneminus(((-(x*c)/(2-c))-x))
  return expo_select(a0, c, k, dbits(cd2::minlog2), dbits(cd2::maxlog2));
}

template <bool F = false>
__device__ __forceinline__ double exp10(double a0)
{
  constexpr uint64_t P[4] = {0x3fa4fd75f3062dd4ull, 0x40277d9474c55934ull, 0x40796b7a050349e4ull,
                             0x40a2b4798e134a01ull};
  constexpr uint64_t Q[4] = {0x3ff0000000000000ull, 0x405545fdce51ca08ull, 0x4093e05eefd67782ull,
                             0x40a03f37650df6e2ull};
  double k = rint(mul(dbits(cd2::invlog10_2), a0));
  double x = nmsub<F>(k, dbits(cd2::log10_2hi), a0);
  x = nmsub<F>(k, dbits(cd2::log10_2lo), x);
  double xx = mul(x, x);
  double px = mul(x, horner<F>(xx, P));
  double x2 = div(px, sub(horner<F>(xx, Q), px));
  double c = add(add(x2, x2), 1.0);                         // oneplus(x2+x2)
  return expo_select(a0, c, k, dbits(cd2::minlog10), dbits(cd2::maxlog10));
}

// d_log.hpp kernel_log (:57-87): returns -(hfsq - s*(hfsq+R) - f), the log of the mantissa
template <bool F>
__device__ __forceinline__ double log_mantissa(double a0, double& dk)
{
  constexpr uint64_t T1[3] = {0x3fc39a09d078c69full, 0x3fcc71c51d8e78afull, 0x3fd999999997fa04ull};
  constexpr uint64_t T2[4] = {0x3fc2f112df3e5244ull, 0x3fc7466496cb03deull, 0x3fd2492494229359ull,
                              0x3fe5555555555593ull};
  unsigned long long u = (unsigned long long)__double_as_longlong(a0);
  long long k = (long long)((u & 0x7ff0000000000000ull) >> 52) - 1022;
  double x = __longlong_as_double((long long)((u & ~0x7ff0000000000000ull) | 0x3fe0000000000000ull));
  bool lt = dbits(cd::sqrt_2o_2) > x;
  k = k + (lt ? -1 : 0);
  double f = sub(add(x, lt ? x : 0.0), 1.0);
  dk = (double)k;
  double s = div(f, add(2.0, f));
  double z = mul(s, s);
  double w = mul(z, z);
  double R = add(mul(z, horner<F>(w, T2)), mul(w, horner<F>(w, T1)));
  double hfsq = mul(0.5, mul(f, f));
  return -sub(sub(hfsq, mul(s, add(hfsq, R))), f);
}

__device__ __forceinline__ double log_finalize(double a0, double y)
{
  y = (a0 < 0.0 || a0 != a0) ? __longlong_as_double(0x7fffffffffffffffll) : y;
  y = (a0 == __longlong_as_double(0x7ff0000000000000ll)) ? a0 : y;
  return (a0 == 0.0) ? __longlong_as_double((long long)0xfff0000000000000ull) : y;
}

template <bool F = false>
__device__ __forceinline__ double log2(double a0)
{
  double dk;
  const double m = log_mantissa<F>(a0, dk);
  return log_finalize(a0, madd<F>(m, dbits(cd::invlog_2), dk));
}

template <bool F = false>
__device__ __forceinline__ double log10(double a0)
{
  double dk;
  const double m = log_mantissa<F>(a0, dk);
  return log_finalize(a0, madd<F>(m, dbits(cd2::invlog_10), mul(dk, dbits(cd2::log_2olog_10))));
}

// --------------------------------------------------- double expm1, log1p
template <bool F = false>
__device__ __forceinline__ double expm1(double a0)
{
  constexpr uint64_t P[6] = {0xBE8AFDB76E09C32Dull, 0x3ED0CFCA86E65239ull, 0xBF14CE199EAADBB7ull,
                             0x3F5A01A019FE5585ull, 0xBFA11111111110F4ull, 0x3ff0000000000000ull};
  double k = rint(mul(dbits(cd::invlog_2), a0));
  double hi = nmsub<F>(k, dbits(cd::log_2hi), a0);
  double lo = mul(k, dbits(cd::log_2lo));
  double x = sub(hi, lo);
  double hxs = mul(mul(x, x), 0.5);
  double r1 = horner<F>(hxs, P);
  double t = nmsub<F>(mul(r1, 0.5), x, 3.0);                 // Three - r1*Half*x
  double e = mul(hxs, div(sub(r1, t), nmsub<F>(x, t, 6.0)));
  double c = sub(sub(hi, x), lo);
  e = sub(sub(mul(x, sub(e, c)), c), hxs);
  long long ik = (long long)k;
  double two2mk = __longlong_as_double((long long)((unsigned long long)(1023 - ik) << 52));
  double ct1 = sub(sub(1.0, two2mk), sub(e, x));
  double ct2 = add(sub(x, add(e, two2mk)), 1.0);
  double y = (k < 20.0) ? ct1 : ct2;
  double r = mul(y, __longlong_as_double((long long)((unsigned long long)(ik + 1023) << 52)));
  r = (a0 > dbits(cd::maxlog)) ? __longlong_as_double(0x7ff0000000000000ll) : r;
  return (a0 < __longlong_as_double(0xc04205966f2b4f19ll)) ? -1.0 : r;   // Logeps
}

template <bool F = false>
__device__ __forceinline__ double log1p(double a0)
{
  double u = add(1.0, a0);
  double r = log<F>(u);
  r = (u != 0.0) ? add(r, div(sub(a0, sub(u, 1.0)), u)) : r;
  return (u == __longlong_as_double(0x7ff0000000000000ll)) ? u : r;
}

// -------------------------------------------------------------- double erfc
// modules/core/euler/include/nt2/euler/functions/simd/common/erfc.hpp:46-89
// kernels: modules/core/euler/include/nt2/euler/functions/details/erf_kernel.hpp:101-163
template <bool F = false>
__device__ __forceinline__ double erfc_abs(double x)
{
  constexpr uint64_t E1P[5] = {0x3f110512d5b20332ull, 0x3f53b7664358865aull, 0x3fa4a59a4f02579cull,
                               0x3fc16500f106c0a5ull, 0x3ff20dd750429b61ull};
  constexpr uint64_t E1Q[5] = {0x3f37ea4332348252ull, 0x3f8166f75999dbd1ull, 0x3fb64536ca92ea2full,
                               0x3fdd0a84eb1ca867ull, 0x3ff0000000000000ull};
  constexpr uint64_t E2P[7] = {0x0ull, 0x3f7cf4cfe0aacbb4ull, 0x3fb2488a6b5cb5e5ull, 0x3fd53dd7a67c7e9full,
                               0x3fec1986509e687bull, 0x3ff54dfe9b258a60ull, 0x3feffffffbbb552bull};
  constexpr uint64_t E2Q[7] = {0x3f89a996639b0d00ull, 0x3fc033c113a7deeeull, 0x3fe307622fcff772ull,
                               0x3ff9e677c2777c3cull, 0x40053b1052dca8bdull, 0x4003adeae79b9708ull,
                               0x3ff0000000000000ull};
  constexpr uint64_t E3P[7] = {0x0ull, 0x3f971d0907ea7a92ull, 0x3fc42210f88b9d43ull, 0x3fe29be1cff90d94ull,
                               0x3ff44744306832aeull, 0x3ff9fa202deb88e5ull, 0x3fefff5a9e697ae2ull};
  constexpr uint64_t E3Q[7] = {0x3fa47bd61bbb3843ull, 0x3fd1d7ab774bb837ull, 0x3ff0cfd4cb6cde9full,
                               0x400315ffdfd5ce91ull, 0x400afd487397568full, 0x400602f24bf3fdb6ull,
                               0x3ff0000000000000ull};
  double xx = mul(x, x);
  double r1;
  if (x < 0.65) {
    r1 = sub(1.0, mul(x, div(horner<F>(xx, E1P), horner<F>(xx, E1Q))));
  } else {
    double ex = exp<F>(-xx);
    if (x < 2.2) r1 = mul(ex, div(horner<F>(x, E2P), horner<F>(x, E2Q)));
    else         r1 = mul(ex, div(horner<F>(x, E3P), horner<F>(x, E3Q)));
  }
  return (x == __longlong_as_double(0x7ff0000000000000ll)) ? 0.0 : r1;
}

template <bool F = false>
__device__ __forceinline__ double erfc(double a0)
{
  double r1 = erfc_abs<F>(fabs(a0));
  return (a0 < 0.0) ? sub(2.0, r1) : r1;
}

template <bool F = false>
__device__ __forceinline__ double normcdf(double a0)
{
  return mul(0.5, erfc<F>(mul(-dbits(cd::sqrt_2o_2), a0)));
}

template <bool F = false>
__device__ __forceinline__ void normcdf_pair(double a0, double& pos, double& neg)
{
  double y = mul(-dbits(cd::sqrt_2o_2), a0);
  double r1 = erfc_abs<F>(fabs(y));
  double two_m = sub(2.0, r1);
  pos = mul(0.5, (y < 0.0) ? two_m : r1);
  neg = mul(0.5, (-y < 0.0) ? two_m : r1);
}

// ---------------------------------------------------- sinh, cosh, tanh
// modules/core/hyperbolic/include/nt2/hyperbolic/functions/: sinh simd/common/sinh.hpp:20-45
// (kernel details/sinh_kernel.hpp), cosh generic/cosh.hpp:20-42, tanh
// simd/common/tanh.hpp:20-48 (kernel details/tanh_kernel.hpp).  The SIMD forms
// select per lane (no pack dependence).  average(a, b) = fma(a, 0.5, b*0.5).
template <class T> struct hyp;
template <> struct hyp<float> {
  static constexpr uint32_t log_2 = 0x3f317218u;
  __device__ static float maxlog() { return fbits(cf::maxlog); }
};
template <> struct hyp<double> {
  static constexpr uint64_t log_2 = 0x3fe62e42fefa39efull;
  __device__ static double maxlog() { return dbits(cd::maxlog); }
};
__device__ __forceinline__ float bits_xor(float v, float s)
{ return __uint_as_float(__float_as_uint(v) ^ (__float_as_uint(s) & 0x80000000u)); }
__device__ __forceinline__ double bits_xor(double v, double s)
{
  return __longlong_as_double(__double_as_longlong(v) ^ (__double_as_longlong(s) & (long long)0x8000000000000000ull));
}

template <bool F, class T> __device__ __forceinline__ T sinh_kernel(T x);
template <> __device__ __forceinline__ float sinh_kernel<false, float>(float x)
{
  constexpr uint32_t P[4] = {0x39559e2fu, 0x3c087bbeu, 0x3e2aaaccu, 0x3f800000u};
  return mul(horner<false>(mul(x, x), P), x);
}
template <> __device__ __forceinline__ float sinh_kernel<true, float>(float x)
{
  constexpr uint32_t P[4] = {0x39559e2fu, 0x3c087bbeu, 0x3e2aaaccu, 0x3f800000u};
  return mul(horner<true>(mul(x, x), P), x);
}
template <bool F> __device__ __forceinline__ double sinh_kernel_d(double x)
{
  constexpr uint64_t P[4] = {0xbfe9435fe8bb3cd6ull, 0xc064773a398ff4feull, 0xc0c694b8c71d6182ull,
                             0xc115782bdbf6ab05ull};
  constexpr uint64_t Q[4] = {0x3ff0000000000000ull, 0xc0715b6096e96484ull, 0x40e1a7ba7ed72245ull,
                             0xc1401a20e4f90044ull};
  const double x2 = mul(x, x);
  return madd<F>(x, div(mul(x2, horner<F>(x2, P)), horner<F>(x2, Q)), x);
}
template <> __device__ __forceinline__ double sinh_kernel<false, double>(double x) { return sinh_kernel_d<false>(x); }
template <> __device__ __forceinline__ double sinh_kernel<true, double>(double x) { return sinh_kernel_d<true>(x); }

template <bool F = false, class T> __device__ __forceinline__ T sinh(T a0)
{
  const T x = fabs(a0);
  T r;
  if (x < T(1)) {
    r = sinh_kernel<F, T>(x);
  } else {
    const bool test1 = x > sub(hyp<T>::maxlog(), (T)(sizeof(T) == 4 ? (T)fbits((uint32_t)hyp<float>::log_2)
                                                                   : (T)dbits(hyp<double>::log_2)));
    const T tmp = exp<F>(mul(x, test1 ? T(0.5) : T(1)));
    const T tmp1 = mul(T(0.5), tmp);
    r = test1 ? mul(tmp1, tmp) : sub(tmp1, mul(T(0.5), div(T(1), tmp)));
  }
  return bits_xor(r, a0);
}
template <bool F = false, class T> __device__ __forceinline__ T cosh(T a0)
{
  const T x = fabs(a0);
  const bool test1 = x > sub(hyp<T>::maxlog(), (T)(sizeof(T) == 4 ? (T)fbits((uint32_t)hyp<float>::log_2)
                                                                 : (T)dbits(hyp<double>::log_2)));
  const T tmp = exp<F>(mul(x, test1 ? T(0.5) : T(1)));
  return test1 ? mul(mul(T(0.5), tmp), tmp) : madd<F>(tmp, T(0.5), mul(div(T(1), tmp), T(0.5)));
}
template <bool F = false> __device__ __forceinline__ float tanh(float a0)
{
  constexpr uint32_t P[5] = {0xbbbaf0eau, 0x3ca9134eu, 0xbd5c1e2du, 0x3e088393u, 0xbeaaaa99u};
  const float x = fabsf(a0);
  float r;
  if (x < 0.625f) {
    const float x2 = mul(x, x);
    r = madd<F>(mul(horner<F>(x2, P), x2), x, x);
  } else {
    r = madd<F>(-2.0f, div(1.0f, add(1.0f, exp<F>(add(x, x)))), 1.0f);
  }
  return bits_xor(r, a0);
}
template <bool F = false> __device__ __forceinline__ double tanh(double a0)
{
  constexpr uint64_t P[3] = {0xbfeedc5baafd6f4bull, 0xc058d26a0e26682dull, 0xc0993ac030580563ull};
  constexpr uint64_t Q[4] = {0x3ff0000000000000ull, 0x405c33f28a581b86ull, 0x40a176fa0e5535faull,
                             0x40b2ec102442040cull};
  const double x = fabs(a0);
  double r;
  if (x < 0.625) {
    const double x2 = mul(x, x);
    r = madd<F>(div(mul(x2, horner<F>(x2, P)), horner<F>(x2, Q)), x, x);
  } else {
    r = madd<F>(-2.0, div(1.0, add(1.0, exp<F>(add(x, x)))), 1.0);
  }
  return bits_xor(r, a0);
}

// coth and sinhc, NT2's SIMD forms (modules/core/hyperbolic/include/nt2/hyperbolic/functions/
// simd/common/coth.hpp:32-48, sinhc.hpp:32-56; kernels details/tanh_kernel.hpp:40-58,
// sinhc_kernel.hpp:25-57); average(a, b) = fma(a, 1/2, b/2); fma(2, r, 1) = 2r + 1.
template <bool F = false> __device__ __forceinline__ float coth(float a0)
{
  constexpr uint32_t P[5] = {0xbbbaf0eau, 0x3ca9134eu, 0xbd5c1e2du, 0x3e088393u, 0xbeaaaa99u};
  const float x = fabsf(a0), x2 = mul(x, x);
  const float r = x < 0.625f ? div(1.0f, madd<F>(mul(horner<F>(x2, P), x2), x, x))
                             : madd<F>(2.0f, div(1.0f, sub(exp<F>(add(x, x)), 1.0f)), 1.0f);
  return bits_xor(r, a0);
}
template <bool F = false> __device__ __forceinline__ double coth(double a0)
{
  constexpr uint64_t P[3] = {0xbfeedc5baafd6f4bull, 0xc058d26a0e26682dull, 0xc0993ac030580563ull};
  constexpr uint64_t Q[4] = {0x3ff0000000000000ull, 0x405c33f28a581b86ull, 0x40a176fa0e5535faull,
                             0x40b2ec102442040cull};
  const double x = fabs(a0), x2 = mul(x, x);
  double r;
  if (x < 0.625) {
    const double q = horner<F>(x2, Q);
    r = div(q, mul(x, madd<F>(horner<F>(x2, P), x2, q)));
  } else {
    r = madd<F>(2.0, div(1.0, sub(exp<F>(add(x, x)), 1.0)), 1.0);
  }
  return bits_xor(r, a0);
}
template <bool F = false, class T> __device__ __forceinline__ T sinhc(T a0)
{
  const T x = fabs(a0);
  T z;
  if constexpr (sizeof(T) == 4) {
    constexpr uint32_t P[4] = {0x39559e2fu, 0x3c087bbeu, 0x3e2aaaccu, 0x3f800000u};
    z = horner<F>(mul(x, x), P);
  } else {
    constexpr uint64_t P[4] = {0xbfe9435fe8bb3cd6ull, 0xc064773a398ff4feull, 0xc0c694b8c71d6182ull,
                               0xc115782bdbf6ab05ull};
    constexpr uint64_t Q[4] = {0x3ff0000000000000ull, 0xc0715b6096e96484ull, 0x40e1a7ba7ed72245ull,
                               0xc1401a20e4f90044ull};
    const T x2 = mul(x, x);
    z = add(T(1), div(mul(x2, horner<F>(x2, P)), horner<F>(x2, Q)));
  }
  if (x < T(1)) return z;
  const T log_2 = sizeof(T) == 4 ? (T)fbits(0x3f317218u) : (T)dbits(0x3fe62e42fefa39efull);
  const bool test1 = x > sub(hyp<T>::maxlog(), log_2);
  const T tmp = exp<F>(mul(x, test1 ? T(0.5) : T(1)));
  const T tmp1 = div(mul(T(0.5), tmp), x);
  const T r = test1 ? mul(tmp1, tmp) : div(madd<F>(tmp, T(0.5), mul(-div(T(1), tmp), T(0.5))), x);
  return x == T(INFINITY) ? x : r;
}

// ------------------------------------------------------ inverse hyperbolic
// atanh and acosh, NT2's SIMD forms (modules/core/hyperbolic/include/nt2/hyperbolic/functions/
// simd/common/atanh.hpp:38-47, acosh.hpp:36-43); NT2's fma(t, tmp, t) is rounded twice in
// the exact form; seladd(c, a, b) = a + (c ? b : 0) is an add on every lane.
template <bool F = false, class T> __device__ __forceinline__ T atanh(T a0)
{
  const T ax = fabs(a0), t = add(ax, ax), z1 = sub(T(1), ax);
  const bool test = ax < T(0.5);
  const T tmp = div(test ? ax : t, z1);
  const T r = mul(T(0.5), log1p<F>(test ? madd<F>(t, tmp, t) : tmp));
  return bits_xor(r, a0);
}
template <bool F = false, class T> __device__ __forceinline__ T acosh(T a0)
{
  const T t = sub(a0, T(1));
  const T oneotwoeps = sizeof(T) == 4 ? (T)fbits(0x4a800000u) : (T)dbits(0x4320000000000000ull);
  const T log_2 = sizeof(T) == 4 ? (T)fbits(0x3f317218u) : (T)dbits(0x3fe62e42fefa39efull);
  const bool test = t > oneotwoeps;
  const T z = test ? a0 : add(t, sqrt_(add(add(t, t), mul(t, t))));
  return add(log1p<F>(z), test ? log_2 : T(0));
}

// -------------------------------------------------------------------- pow
// pow(a0, a1) for floating a0 and a1, NT2's SIMD form:
// modules/core/exponential/include/nt2/exponential/functions/simd/common/pow.hpp:29-37 over
// pow_abs (simd/common/pow_abs.hpp:72-131), the cephes algorithm: log2|a0| from a 2^(-i/16)
// table and a rational (double) or polynomial (float) correction, the product with a1 split
// into multiples of 1/16 to keep it exact, and 2^(product) back through the same table
// (details/pow_kernel.hpp).  The scalar form (scalar/pow.hpp, scalar/pow_abs.hpp) runs the
// same kernel and returns the same values for the same special cases.  frexp and ldexp are
// Boost.SIMD's (boost/simd/ieee/functions/simd/common/frexp.hpp:42-67, ldexp.hpp:55-70).
// The tables are 2^(-i/16) rounded to the type (A) and, for even i, the rounding residual
// 2^(-i/16) - A[i] (B, indexed by i/2); they are read through the L1 (a warp's indices fall
// in one or two 128-byte lines).
#define NT2CUDA_POW_AF                                                                                          \
  0x3f800000u, 0x3f75257du, 0x3f6ac0c7u, 0x3f60ccdfu, 0x3f5744fdu, 0x3f4e248cu, 0x3f45672au, 0x3f3d08a4u, 0x3f3504f3u, \
      0x3f2d583fu, 0x3f25fed7u, 0x3f1ef532u, 0x3f1837f0u, 0x3f11c3d3u, 0x3f0b95c2u, 0x3f05aac3u, 0x3f000000u
#define NT2CUDA_POW_AD                                                                                          \
  0x3ff0000000000000ull, 0x3feea4afa2a490daull, 0x3fed5818dcfba487ull, 0x3fec199bdd85529cull, 0x3feae89f995ad3adull, \
      0x3fe9c49182a3f090ull, 0x3fe8ace5422aa0dbull, 0x3fe7a11473eb0187ull, 0x3fe6a09e667f3bcdull,                 \
      0x3fe5ab07dd485429ull, 0x3fe4bfdad5362a27ull, 0x3fe3dea64c123422ull, 0x3fe306fe0a31b715ull,                 \
      0x3fe2387a6e756238ull, 0x3fe172b83c7d517bull, 0x3fe0b5586cf9890full, 0x3fe0000000000000ull
static __device__ const uint32_t kPowAf[17] = {NT2CUDA_POW_AF};
static __device__ const uint32_t kPowBf[9] = {0x00000000u, 0xb1c116deu, 0xb254a58au, 0x318aa837u, 0x324fe77au,
                                              0xb2ac9d5eu, 0x32a31b71u, 0xb1e0aba1u, 0x00000000u};
static __device__ const uint64_t kPowAd[17] = {NT2CUDA_POW_AD};
static __device__ const uint64_t kPowBd[9] = {0x0000000000000000ull, 0x3c72ed02d75b3707ull, 0x3c87a1cd345dcc81ull,
                                              0x3c86e9f156864b27ull, 0xbc8bdd3413b26456ull, 0x3c6d4397afec42e2ull,
                                              0x3c76f46ad23182e4ull, 0xbc719041b9d78a76ull, 0x0000000000000000ull};

__device__ __forceinline__ float pow_a(float, int i) { return __uint_as_float(__ldg(&kPowAf[i])); }
__device__ __forceinline__ float pow_b(float, int i) { return __uint_as_float(__ldg(&kPowBf[i])); }
__device__ __forceinline__ double pow_a(double, int i)
{ return __longlong_as_double((long long)__ldg(reinterpret_cast<const unsigned long long*>(&kPowAd[i]))); }
__device__ __forceinline__ double pow_b(double, int i)
{ return __longlong_as_double((long long)__ldg(reinterpret_cast<const unsigned long long*>(&kPowBd[i]))); }

template <class T> struct powc;
template <> struct powc<float> {
  using U = uint32_t;
  static constexpr int nbm = 23, maxe = 127, mine = -126, lime = 128;
  static constexpr U expmask = 0x7f800000u, half = 0x3f000000u, smallest = 0x00800000u;
  static constexpr U log2_em1 = 0x3ee2a8edu, large = 0x44ffe000u, low = 0xc5160000u;
  __device__ static float bits(U u) { return __uint_as_float(u); }
  __device__ static U ubits(float v) { return __float_as_uint(v); }
  __device__ static float twotonmb() { return 8388608.0f; }
};
template <> struct powc<double> {
  using U = uint64_t;
  static constexpr int nbm = 52, maxe = 1023, mine = -1022, lime = 1024;
  static constexpr U expmask = 0x7ff0000000000000ull, half = 0x3fe0000000000000ull,
                     smallest = 0x0010000000000000ull;
  static constexpr U log2_em1 = 0x3fdc551d94ae0bf8ull, large = 0x40cfff8000000000ull, low = 0xc0d0c7c000000000ull;
  __device__ static double bits(U u) { return __longlong_as_double((long long)u); }
  __device__ static U ubits(double v) { return (U)__double_as_longlong(v); }
  __device__ static double twotonmb() { return 4503599627370496.0; }
};

// Boost.SIMD frexp: mantissa in [0.5, 1), denormals scaled by 2^nbm first; Inf/NaN keep a
// mantissa that is not finite (r0 + a0) and exponent 0.
template <class T> __device__ __forceinline__ T pow_frexp(T a0, int& e)
{
  using C = powc<T>;
  const bool den = fabs(a0) < C::bits(C::smallest) && a0 != T(0);
  const T aa0 = den ? mul(C::twotonmb(), a0) : a0;
  const typename C::U b = C::ubits(aa0);
  int r1 = (int)((b & C::expmask) >> C::nbm) - (C::maxe - 1);
  const T r0 = C::bits((b & ~C::expmask) | C::half);
  const bool test0 = aa0 != T(0), test1 = r1 > C::lime;
  r1 = (!test1 && test0) ? r1 : 0;
  e = r1 - (den ? C::nbm : 0);
  return test0 ? (test1 ? add(r0, aa0) : r0) : T(0);
}
// Boost.SIMD ldexp: (a0 * 2^e) * f with f = 2^mine for exponents below mine and 2 for e = lime.
// The exponent bits are built with an unsigned shift (e stays in [-2000, 1100] for the results
// that pow keeps).
template <class T> __device__ __forceinline__ T pow_ldexp(T a0, int e)
{
  using C = powc<T>;
  const bool den = e < C::mine;
  e = den ? e - C::mine : e;
  T f = den ? C::bits(C::smallest) : T(1);
  const bool test = e == C::lime;
  f = test ? add(f, T(1)) : f;
  e = test ? e - 1 : e;
  const T s = C::bits((typename C::U)(unsigned)(e + C::maxe) << C::nbm);
  return mul(mul(a0, s), f);
}
template <class T> __device__ __forceinline__ T pow_reduc(T x) { return mul(T(0.0625), floor(mul(T(16), x))); }

// pow_kernel::select: i in 0..16 from x in [0.5, 1); x <- (x - A[i] - B[i/2]) / A[i].  The
// indices it reads are 9, 13, 3..15 (odd), 1 and i itself, all inside the table.
template <class T> __device__ __forceinline__ T pow_ac(int i);  // A[i] for a constant i
template <> __device__ __forceinline__ float pow_ac<float>(int i)
{
  constexpr uint32_t A[17] = {NT2CUDA_POW_AF};
  return __uint_as_float(A[i]);
}
template <> __device__ __forceinline__ double pow_ac<double>(int i)
{
  constexpr uint64_t A[17] = {NT2CUDA_POW_AD};
  return __longlong_as_double((long long)A[i]);
}
template <class T> __device__ __forceinline__ int pow_index(T x)
{
  // The search compares x with A[9], then A[5] or A[13], then one of A[3], A[7],
  // A[11], A[15], then A[1]: values picked from constants instead of table reads.
  int i = 1;
  i = (x <= pow_ac<T>(9)) ? 9 : i;
  i = (x <= (i == 9 ? pow_ac<T>(13) : pow_ac<T>(5))) ? i + 4 : i;
  const T a2 = i == 1 ? pow_ac<T>(3) : (i == 5 ? pow_ac<T>(7) : (i == 9 ? pow_ac<T>(11) : pow_ac<T>(15)));
  i = (x <= a2) ? i + 2 : i;
  i = (x >= pow_ac<T>(1)) ? -1 : i;
  return i + 1;
}
template <class T> __device__ __forceinline__ int pow_select(T& x)
{
  const int i = pow_index(x);
  const T tmp = pow_a(x, i);
  x = sub(x, tmp);
  x = sub(x, pow_b(x, i >> 1));
  x = div(x, tmp);
  return i;
}

template <bool F> __device__ __forceinline__ float pow1(float x, float z)
{
  constexpr uint32_t P[4] = {0xbe2a61b2u, 0x3e4d2fa3u, 0xbe800015u, 0x3eaaaaa3u};
  return mul(mul(z, x), horner<F>(x, P));
}
template <bool F> __device__ __forceinline__ double pow1(double x, double z)
{
  constexpr uint64_t P[4] = {0x3fdfdb997f5b5cf0ull, 0x400dddefea9edf15ull, 0x401eccbd7f78eb6full, 0x4012aa83b65c9b74ull};
  constexpr uint64_t Q[5] = {0x3ff0000000000000ull, 0x4022aab49b20914eull, 0x403bffff41c1c9f5ull,
                             0x4040ccbc1b176402ull, 0x402bffc5918ae92eull};
  return mul(x, div(mul(z, horner<F>(x, P)), horner<F>(x, Q)));
}
template <bool F> __device__ __forceinline__ float pow2(float x)
{
  constexpr uint32_t P[4] = {0x3c1a49bcu, 0x3d634d38u, 0x3e75fde1u, 0x3f317218u};
  return horner<F>(x, P);
}
template <bool F> __device__ __forceinline__ double pow2(double x)
{
  constexpr uint64_t P[7] = {0x3eef6307d7f2937full, 0x3f242fbe60fc9259ull, 0x3f55d87ec84aef1dull,
                             0x3f83b2ab6ef133b7ull, 0x3fac6b08d7041a92ull, 0x3fcebfbdff82c56dull,
                             0x3fe62e42fefa39efull};
  return horner<F>(x, P);
}

template <bool F = false, class T> __device__ __forceinline__ T pow_abs(T a0, T a1)
{
  using C = powc<T>;
  const T ax = fabs(a0);
  int e;
  T x = pow_frexp(ax, e);
  int i = pow_select(x);
  T z = mul(x, x);
  T w = pow1<F>(x, z);
  w = madd<F>(T(-0.5), z, w);
  w = madd<F>(C::bits(C::log2_em1), w, w);
  z = madd<F>(C::bits(C::log2_em1), x, w);
  z = add(z, x);
  w = madd<F>((T)(-i), T(0.0625), (T)e);
  const T ya = pow_reduc(a1);
  const T yb = sub(a1, ya);
  T W = madd<F>(z, a1, mul(w, yb));
  T Wa = pow_reduc(W);
  T Wb = sub(W, Wa);
  W = madd<F>(w, ya, Wa);
  Wa = pow_reduc(W);
  const T u = sub(W, Wa);
  W = add(Wb, u);
  Wb = pow_reduc(W);
  w = mul(T(16), add(Wa, Wb));
  const bool inf_ret = w > C::bits(C::large), zer_ret = w < C::bits(C::low);
  // toint(w): every w outside [low, large] (NaN aside) is replaced below, so the
  // conversion is clamped to keep the integer steps defined; in range it truncates as NT2's.
  e = (int)fmin(fmax(w, T(-32768)), T(32768));
  Wb = sub(W, Wb);
  const bool test = Wb > T(0);
  e = test ? e + 1 : e;
  Wb = test ? sub(Wb, T(0.0625)) : Wb;
  z = mul(pow2<F>(Wb), Wb);
  i = (e > 0) ? e / 16 + 1 : e / 16;
  e = i * 16 - e;  // 0..16 for every w that is kept
  w = pow_a(z, min(max(e, 0), 16));
  z = madd<F>(w, z, w);
  z = pow_ldexp(z, i);
  const bool gtax1 = ax > T(1);
  const T inf = C::bits(C::expmask);
  if (a1 == inf) z = gtax1 ? inf : T(0);
  if (a1 == -inf) z = gtax1 ? T(0) : inf;
  if (ax == inf) z = a1 > T(0) ? inf : (a1 < T(0) ? T(0) : T(1));
  if (zer_ret) z = T(0);
  if (inf_ret) z = inf;
  if (ax == T(1)) z = ax;
  return a0 == T(0) ? (a1 == T(0) ? T(1) : T(0)) : z;
}

// Boost.SIMD is_flint (frac(x) == 0, frac = x - trunc(x), NaN for Inf and NaN) and is_odd
// (is_flint((x - 1) / 2)): boost/simd/predicates/functions/simd/common/{is_flint,is_odd,is_even}.hpp.
template <class T> __device__ __forceinline__ bool is_flint(T x) { return isfinite(x) && sub(x, trunc(x)) == T(0); }

template <bool F = false, class T> __device__ __forceinline__ T pow(T a0, T a1)
{
  const bool ltz = a0 < T(0);
  T z = pow_abs<F>(a0, a1);
  if (ltz && is_flint(mul(sub(a1, T(1)), T(0.5)))) z = -z;
  return (ltz && !is_flint(a1)) ? T(NAN) : z;
}

// ------------------------------------------------- rest of the exp family
// cbrt, NT2's SIMD forms (modules/core/exponential/include/nt2/exponential/functions/simd/
// common/cbrt.hpp:36-89 double, :91-142 float): Boost.SIMD fast_frexp (no special cases), a
// degree-4 polynomial, the exponent divided by 3 with 2^(1/3) or 2^(2/3) for the remainder,
// fast_ldexp, then Newton steps (two in double, one in float); zeros and infinities are
// returned as they are.
__device__ __forceinline__ int cbrt_split(int e, int& rem)
{
  int e1 = e < 0 ? -e : e;
  rem = e1 - (e1 / 3) * 3;
  e1 /= 3;
  return e > 0 ? e1 : (e < 0 ? -e1 : 0);  // negate(e1, e): e1 with the sign of e, 0 for 0
}
template <bool F = false> __device__ __forceinline__ float cbrt(float a0)
{
  constexpr uint32_t P[5] = {0xbe09e49au, 0x3f0bf0feu, 0xbf745265u, 0x3f91eb77u, 0x3ece0609u};
  float z = fabsf(a0);
  const bool den = z < fbits(0x00800000u);
  z = den ? mul(z, 8388608.0f) : z;
  const float f = den ? fbits(0x3ba14518u) : 1.0f;  // 2^(-23/3)
  const uint32_t b = __float_as_uint(z);
  int e = (int)((b & 0x7f800000u) >> 23) - 126;    // e <= 129 (Inf/NaN): e / 3 stays small
  float x = fbits((b & ~0x7f800000u) | 0x3f000000u);
  x = horner<F>(x, P);
  const bool flag = e >= 0;
  int rem;
  e = cbrt_split(e, rem);
  float fact = rem == 1 ? (flag ? fbits(0x3fa14518u) : fbits(0x3f4b2ff5u)) : 1.0f;
  fact = rem == 2 ? (flag ? fbits(0x3fcb2ff5u) : fbits(0x3f214518u)) : fact;
  x = mul(mul(x, fact), fbits((uint32_t)(e + 127) << 23));
  x = sub(x, mul(sub(x, div(z, mul(x, x))), fbits(0x3eaaaaabu)));
  x = mul(__uint_as_float(__float_as_uint(x) | (__float_as_uint(a0) & 0x80000000u)), f);
  return (a0 == 0.0f || isinf(a0)) ? a0 : x;
}
template <bool F = false> __device__ __forceinline__ double cbrt(double a0)
{
  constexpr uint64_t P[5] = {0xbfc13c93386fdff6ull, 0x3fe17e1fc7e59d58ull, 0xbfee8a4ca3ba37b8ull,
                             0x3ff23d6ee505873aull, 0x3fd9c0c12122a4feull};
  double z = fabs(a0);
  const bool den = z < dbits(0x0010000000000000ull);
  z = den ? mul(z, 4503599627370496.0) : z;
  const double f = den ? dbits(0x3ed428a2f98d7286ull) : 1.0;  // 2^(-52/3)
  const uint64_t b = (uint64_t)__double_as_longlong(z);
  int e = (int)((b & 0x7ff0000000000000ull) >> 52) - 1022;
  double x = dbits((b & ~0x7ff0000000000000ull) | 0x3fe0000000000000ull);
  x = horner<F>(x, P);
  const bool flag = e >= 0;
  int rem;
  e = cbrt_split(e, rem);
  double fact = rem == 1 ? (flag ? dbits(0x3ff428a2f98d728bull) : dbits(0x3fe965fea53d6e3dull)) : 1.0;
  fact = rem == 2 ? (flag ? dbits(0x3ff965fea53d6e3dull) : dbits(0x3fe428a2f98d728bull)) : fact;
  x = mul(mul(x, fact), dbits((uint64_t)(e + 1023) << 52));
  const double third = dbits(0x3fd5555555555555ull);
  x = sub(x, mul(sub(x, div(z, mul(x, x))), third));
  x = sub(x, mul(sub(x, div(z, mul(x, x))), third));
  x = mul(dbits((uint64_t)__double_as_longlong(x) | ((uint64_t)__double_as_longlong(a0) & 0x8000000000000000ull)), f);
  return (a0 == 0.0 || isinf(a0)) ? a0 : x;
}

// sqrt1pm1(x) = sqrt(1+x) - 1 (generic/sqrt1pm1.hpp:27-33)
template <bool F = false, class T> __device__ __forceinline__ T sqrt1pm1(T a0)
{
  const T t = sqrt_(add(a0, T(1)));
  return fabs(a0) < T(0.5) ? div(a0, add(t, T(1))) : sub(t, T(1));
}
// exprecneg(x) = exp(-1/x), exprecnegc(x) = -expm1(-1/x) (generic/exprecneg.hpp:27,
// generic/exprecnegc.hpp:27; rec is the IEEE quotient 1/x)
template <bool F = false, class T> __device__ __forceinline__ T exprecneg(T a0) { return exp<F>(-div(T(1), a0)); }
template <bool F = false, class T> __device__ __forceinline__ T exprecnegc(T a0) { return -expm1<F>(-div(T(1), a0)); }

// expx2(x) = exp(x^2) and expx2(x, s) = exp(sign(s) x^2) (simd/common/expx2.hpp:31-50, :52-74):
// x^2 = u + u1 with u = m^2, m a multiple of Expx2c1 (32 float, 128 double) near |x|.
template <class T> __device__ __forceinline__ T expx2_c1() { return sizeof(T) == 4 ? T(32) : T(128); }
template <bool F = false, class T> __device__ __forceinline__ T expx2(T a0)
{
  const T x = fabs(a0);
  const T m = mul(expx2_c1<T>(), floor(madd<F>(div(T(1), expx2_c1<T>()), x, T(0.5))));
  const T f = sub(x, m);
  const T u = mul(m, m);
  const T u1 = madd<F>(add(m, m), f, mul(f, f));
  const T inf = T(INFINITY);
  const T r = add(u, u1) > hyp<T>::maxlog() ? inf : mul(exp<F>(u), exp<F>(u1));
  return x == inf ? x : r;
}
template <bool F = false, class T> __device__ __forceinline__ T expx2(T a0, T s)
{
  const T sgn = signbit(s) ? T(-1) : T(1);  // signnz: -1 for -0
  const T x = mul(a0, sgn);
  const T m = mul(expx2_c1<T>(), floor(madd<F>(div(T(1), expx2_c1<T>()), x, T(0.5))));
  const T f = sub(x, m);
  const T u = mul(sgn, mul(m, m));
  const T u1 = mul(sgn, madd<F>(add(m, m), f, mul(f, f)));
  const T inf = T(INFINITY);
  const T r = add(u, u1) > hyp<T>::maxlog() ? inf : mul(exp<F>(u), exp<F>(u1));
  return x == inf ? x : r;
}

// logspace_add(a, b) = log(exp(a) + exp(b)), logspace_sub(a, b) = log(exp(a) - exp(b))
// (simd/common/logspace_add.hpp:27-36, logspace_sub.hpp:27-35; the SIMD forms evaluate both
// branches of logspace_sub and select, the value is the selected one's)
template <bool F = false, class T> __device__ __forceinline__ T logspace_add(T a0, T a1)
{
  const T t = -fabs(sub(a0, a1));
  const T r = add(a0 > a1 ? a0 : a1, log1p<F>(exp<F>(t)));
  return isnan(t) ? add(a0, a1) : r;
}
template <bool F = false, class T> __device__ __forceinline__ T logspace_sub(T a0, T a1)
{
  const T x = sub(a1, a0);
  const T log_2 = sizeof(T) == 4 ? (T)fbits(0x3f317218u) : (T)dbits(0x3fe62e42fefa39efull);
  const T t = x > -log_2 ? log<F>(-expm1<F>(x)) : log1p<F>(-exp<F>(x));
  return add(a0, t);
}

// hypot, Boost.SIMD's SIMD form (boost/simd/arithmetic/functions/simd/common/hypot.hpp:33-49):
// e = exponent(max(|a0|, |a1|)) -- 0 for Inf and NaN, the biased exponent minus Maxexponent
// otherwise (so -Maxexponent for zeros and denormals) -- clamped to [Minexponent,
// Maxexponentm1]; both scaled by 2^-e with Boost.SIMD's ldexp, squared, added, square-rooted,
// scaled back; Inf where one argument is NaN and the other infinite.
template <class T> __device__ __forceinline__ T hypot(T a0, T a1)
{
  using C = powc<T>;
  const T r = fabs(a0), i = fabs(a1), m = i > r ? i : r;
  int e = isfinite(m) ? (int)((C::ubits(m) & C::expmask) >> C::nbm) - (m != T(0) ? C::maxe : 0) : 0;
  e = min(max(e, C::mine), C::maxe - 1);
  const T a = pow_ldexp(r, -e), b = pow_ldexp(i, -e);
  const T res = pow_ldexp(sqrt_(add(mul(a, a), mul(b, b))), e);
  return ((isnan(a0) && isinf(a1)) || (isnan(a1) && isinf(a0))) ? T(INFINITY) : res;
}
// asinh, NT2's SIMD forms (modules/core/hyperbolic/include/nt2/hyperbolic/functions/simd/common/
// asinh.hpp:46-64 double: log1p of x + x^2/(1 + hypot(1, x)); :66-94 float: a polynomial below
// 1/2, else log of average(x, hypot(1, x)) plus log 2; average(a, b) = fma(a, 1/2, b/2))
template <bool F = false> __device__ __forceinline__ float asinh(float a0)
{
  constexpr uint32_t P[5] = {0x3ca4d6e6u, 0xbd2ee581u, 0x3d9949b1u, 0xbe2aa9adu, 0x3f800000u};
  const float x = fabsf(a0), x2 = mul(x, x);
  const float z = mul(horner<F>(x2, P), x);
  const float tmp = x > fbits(0x453504f3u) ? x : madd<F>(x, 0.5f, mul(hypot(1.0f, x), 0.5f));
  const float r = x < 0.5f ? z : add(log<F>(tmp), fbits(0x3f317218u));
  return bits_xor(r, a0);
}
template <bool F = false> __device__ __forceinline__ double asinh(double a0)
{
  const double x = fabs(a0);
  const bool test = x > dbits(0x4190000000000000ull);
  double z = test ? sub(x, 1.0) : add(x, div(mul(x, x), add(1.0, hypot(1.0, x))));
  z = x == INFINITY ? x : z;
  return bits_xor(add(log1p<F>(z), test ? dbits(0x3fe62e42fefa39efull) : 0.0), a0);
}

}  // namespace math
}  // namespace nt2cuda

// ---------------------------------------------------------------------------
// Fast variants (precision mode 2): hardware FMA, the GB300 special-function
// unit for 2^x, log2 x, rsqrt and reciprocals (PTX ex2.approx / lg2.approx),
// and a branch-free erfc for normcdf.  Their distance to the exact NT2 forms
// and to FP64 is measured by the parity tests; they are not bit-exact.
namespace nt2cuda {
namespace math {
namespace fast {

__device__ __forceinline__ float ex2(float x)
{
  float r;
  asm("ex2.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float lg2(float x)
{
  float r;
  asm("lg2.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// exp(x): NT2's Cody-Waite reduction x = k*ln2 + f (FMA form), then 2^(f*log2e)
// on the special-function unit and the exponent scale by integer add; the
// reduced argument keeps ex2.approx's error at a few ulp over the whole range.
__device__ __forceinline__ float exp(float a0)
{
  const float k = rintf(__fmul_rn(fbits(cf::invlog_2), a0));
  float f = __fmaf_rn(-k, fbits(cf::log_2hi), a0);
  f = __fmaf_rn(-k, fbits(cf::log_2lo), f);
  const float p = ex2(__fmul_rn(f, fbits(cf::invlog_2)));
  const int ik = (int)k;
  // 2^k in two halves so that k down to -149 and up to 127 scale exactly
  const float s1 = __int_as_float((unsigned)((ik >> 1) + 127) << 23);
  const float s2 = __int_as_float((unsigned)((ik - (ik >> 1)) + 127) << 23);
  float r = __fmul_rn(__fmul_rn(p, s1), s2);
  r = (a0 <= fbits(cf::minlog)) ? 0.0f : r;
  r = (a0 >= fbits(cf::maxlog)) ? __int_as_float(0x7f800000) : r;
  return (a0 != a0) ? a0 : r;
}

// exp(x) for moderate |x| (exp(-r*T), exp(-x^2) inside erfc): 2^(x*log2e) on
// the special-function unit; the rounding of x*log2e adds |x|*2^-24*log2e of
// relative error (about 1e-6 at |x| = 10, where exp(-x) is 4.5e-5).
__device__ __forceinline__ float exp_small(float x)
{
  return ex2(__fmul_rn(x, 1.4426950408889634f));
}

// log(x) = log2(x) * ln2 on the special-function unit (absolute error of a few
// 1e-8 near 1, relative error of a few ulp elsewhere); NT2's special values.
__device__ __forceinline__ float log(float a0)
{
  float r = __fmul_rn(lg2(a0), 0.69314718055994530942f);
  r = (a0 < 0.0f || a0 != a0) ? __int_as_float(0x7fffffff) : r;
  r = (a0 == __int_as_float(0x7f800000)) ? a0 : r;
  return (a0 == 0.0f) ? __int_as_float(0xff800000) : r;
}

// erfc(|a|) with NT2's two polynomials (erf_kernel.hpp:48-85) in FMA form;
// x/(1+x) by reciprocal (1+x >= 1).
__device__ __forceinline__ float erfc_abs(float x)
{
  constexpr uint32_t P2[11] = {0xc0283611u, 0x40d67e3bu, 0xc0cd1a85u, 0x4050b063u,
                               0xbfaea865u, 0x3e2006f0u, 0x3e1175c7u, 0x3ec4ca6eu,
                               0x3e243828u, 0xbf918a62u, 0x3f0a0e8bu};
  constexpr uint32_t P3[9] = {0x41aa8e55u, 0x401b5680u, 0xc010d956u, 0x3f2cff3bu,
                              0xc016c985u, 0xbffc9284u, 0xbfa11698u, 0xbe036d7eu, 0x3f7ffffeu};
  const float z = __fdividef(x, __fadd_rn(1.0f, x));
  float r1;
  if (x < fbits(cf::twothird)) {
    r1 = __fmul_rn(__fsub_rn(1.0f, z), horner<true>(z, P3));
  } else {
    r1 = __fmul_rn(exp_small(-__fmul_rn(x, x)), horner<true>(__fsub_rn(z, 0.4f), P2));
  }
  return (x == __int_as_float(0x7f800000)) ? 0.0f : r1;
}

// erfc(x) for x >= 0 without branches: the Chebyshev fit of Press, Teukolsky,
// Vetterling and Flannery, Numerical Recipes in C (2nd ed., section 6.2,
// erfcc), erfc(x) ~ t*exp(-x^2 + P(t)) with t = 1/(1 + x/2) and a degree-9 P,
// fractional error below 1.2e-7 for every x >= 0.  One reciprocal, ten FMAs
// and one 2^x, and no divergence between the small- and large-argument
// regions that NT2's two polynomials need.
__device__ __forceinline__ float erfc_abs_nr(float x)
{
  const float t = __fdividef(1.0f, __fmaf_rn(0.5f, x, 1.0f));
  float p = 0.17087277f;
  p = __fmaf_rn(p, t, -0.82215223f);
  p = __fmaf_rn(p, t, 1.48851587f);
  p = __fmaf_rn(p, t, -1.13520398f);
  p = __fmaf_rn(p, t, 0.27886807f);
  p = __fmaf_rn(p, t, -0.18628806f);
  p = __fmaf_rn(p, t, 0.09678418f);
  p = __fmaf_rn(p, t, 0.37409196f);
  p = __fmaf_rn(p, t, 1.00002368f);
  p = __fmaf_rn(p, t, -1.26551223f);
  return __fmul_rn(t, exp_small(__fmaf_rn(-x, x, p)));
}

__device__ __forceinline__ void normcdf_pair(float a0, float& pos, float& neg)
{
  const float y = __fmul_rn(-fbits(cf::sqrt_2o_2), a0);
  const float r1 = erfc_abs_nr(fabsf(y));
  const float two_m = __fsub_rn(2.0f, r1);
  pos = __fmul_rn(0.5f, (y < 0.0f) ? two_m : r1);
  neg = __fmul_rn(0.5f, (-y < 0.0f) ? two_m : r1);
}

__device__ __forceinline__ void fastnormcdf_pair(float a0, float& pos, float& neg)
{
  constexpr uint32_t P[5] = {0x3faa466fu, 0xbfe91eeau, 0x3fe40778u, 0xbeb68f87u, 0x3ea385fau};
  const float l = fabsf(a0);
  const float k = __fdividef(1.0f, __fmaf_rn(0.2316419f, l, 1.0f));
  float w = horner<true>(k, P);
  w = __fmul_rn(w, __fmul_rn(__fmul_rn(k, fbits(cf::invsqrt_2pi)), exp_small(__fmul_rn(-__fmul_rn(l, l), 0.5f))));
  const float om = __fsub_rn(1.0f, w);
  pos = (a0 > 0.0f) ? om : w;
  neg = (-a0 > 0.0f) ? om : w;
}

}  // namespace fast
}  // namespace math
}  // namespace nt2cuda
