/*
 * nt2_oracle_trig.c -- CPU restatement of NT2's sine, cosine and tangent
 * (sin, cos, tan in radians; sinpi, cospi) and of asin, acos, atan, for
 * float and double.
 *
 * TEST INFRASTRUCTURE ONLY, like nt2_oracle.c: the parity checker of the
 * CUDA evaluator, never called by the product path.
 *
 * Paths are relative to NT2's modules/core/trigonometric/include/nt2/trigonometric/.
 *
 * NT2 evaluates a transform in packs of N lanes from the start of the range
 * and finishes the last n % N elements one at a time
 * (modules/core/base/include/nt2/core/functions/simd/transform.hpp:40-48).
 * Its radian reduction picks ONE method for a whole pack from the pack's
 * largest |x| (functions/scalar/impl/trigo/trig_reduction.hpp:46-160; the
 * `big_` mode of functions/scalar/impl/selection_tags.hpp:55-61):
 *   level 0  all |x| <= pi/4        no reduction
 *   level 1  all |x| <= pi/2        rem_pio2_straight (functions/generic/rem_pio2_straight.hpp)
 *   level 2  all |x| <= 20 pi       rem_pio2_cephes   (functions/generic/rem_pio2_cephes.hpp)
 *   level 3  all |x| <= Medium_pi   rem_pio2_medium   (functions/generic/rem_pio2_medium.hpp);
 *                                   Medium_pi is 2^6 pi for float, 2^18 pi for double
 *   level 4  float, all |x| <= 2^18 pi: each half of the pack is converted to
 *            double and reduced by the double chain (trig_reduction.hpp:161-183)
 *   level 5  rem_pio2 lane by lane (functions/scalar/rem_pio2.hpp: fdlibm's
 *            __ieee754_rem_pio2f :83-232 and __ieee754_rem_pio2 :484-622)
 * so a lane's result depends on the other lanes of its pack.  `pack` below
 * is N (1 = NT2's scalar code, 4 floats / 2 doubles = 128-bit SIMD).
 *
 * Lanes that reach fdlibm's __kernel_rem_pio2f / __kernel_rem_pio2 (float
 * |x| > 2^7 pi/2 at level 5, double |x| > 2^19 pi/2) are reduced here by an
 * exact Payne-Hanek reduction (224 bits of 2/pi, one rounding).  fdlibm's
 * kernels sum their partial products in float/double and may differ in the
 * last bit of the reduced argument: parity for those lanes is unpinned to
 * that bit.  Everything else follows NT2 operation by operation; the
 * polynomials are functions/simd/common/impl/trigo/{f,d}_trig_evaluation.hpp
 * with NT2's unfused fma (the file is built with -ffp-contract=off).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

static inline float tfb(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t tbf(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline double tdb(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static inline uint64_t tbd(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

/* ------------------------------------------------------------ constants -- */
/* Bit patterns of the BOOST_SIMD_CONSTANT_REGISTER lines in the constants headers. */
#define F_PIO4    0x3f490fdbu
#define F_PIO2    0x3fc90fdbu
#define F_20PI    0x427b53d1u
#define F_MEDPI   0x43490fdbu   /* 2^6 pi */
#define F_DMPI    0x49490fdbu   /* 2^18 pi */
#define F_PI      0x40490fdbu
#define F_TWOOPI  0x3f22f983u
#define F_INVPIO2 0x3f22f984u
#define F_PIO2_1  0x3fc90f80u
#define F_PIO2_2  0x37354400u
#define F_PIO2_3  0x2e85a300u
#define F_PIO2_1T 0x37354443u
#define F_PIO2_2T 0x2e85a308u
#define F_PIO2_3T 0x248d3132u

#define D_PIO4    0x3fe921fb54442d18ull
#define D_PIO2    0x3ff921fb54442d18ull
#define D_20PI    0x404f6a7a2955385eull
#define D_MEDPI   0x412921fb54442d18ull   /* 2^18 pi */
#define D_PI      0x400921fb54442d18ull
#define D_TWOOPI  0x3fe45f306dc9c883ull
#define D_INVPIO2 0x3fe45f306dc9c883ull
#define D_PIO2_1  0x3ff921fb54400000ull
#define D_PIO2_2  0x3dd0b4611a600000ull
#define D_PIO2_3  0x3ba3198a2e000000ull
#define D_PIO2_1T 0x3dd0b4611a626331ull
#define D_PIO2_2T 0x3ba3198a2e037073ull
#define D_PIO2_3T 0x397b839a252049c1ull

/* High bits of n*pi/2, n = 1..32 (float: bit pattern with the low 8 bits
 * cleared; double: high word), the "no cancellation" test of fdlibm's
 * medium branch. */
static const uint32_t NPIO2_HW_F[32] = {
  0x3fc90f00u, 0x40490f00u, 0x4096cb00u, 0x40c90f00u, 0x40fb5300u, 0x4116cb00u, 0x412fed00u, 0x41490f00u,
  0x41623100u, 0x417b5300u, 0x418a3a00u, 0x4196cb00u, 0x41a35c00u, 0x41afed00u, 0x41bc7e00u, 0x41c90f00u,
  0x41d5a000u, 0x41e23100u, 0x41eec200u, 0x41fb5300u, 0x4203f200u, 0x420a3a00u, 0x42108300u, 0x4216cb00u,
  0x421d1400u, 0x42235c00u, 0x4229a500u, 0x422fed00u, 0x42363600u, 0x423c7e00u, 0x4242c700u, 0x42490f00u};
static const uint32_t NPIO2_HW_D[32] = {
  0x3ff921fbu, 0x400921fbu, 0x4012d97cu, 0x401921fbu, 0x401f6a7au, 0x4022d97cu, 0x4025fdbbu, 0x402921fbu,
  0x402c463au, 0x402f6a7au, 0x4031475cu, 0x4032d97cu, 0x40346b9cu, 0x4035fdbbu, 0x40378fdbu, 0x403921fbu,
  0x403ab41bu, 0x403c463au, 0x403dd85au, 0x403f6a7au, 0x40407e4cu, 0x4041475cu, 0x4042106cu, 0x4042d97cu,
  0x4043a28cu, 0x40446b9cu, 0x404534acu, 0x4045fdbbu, 0x4046c6cbu, 0x40478fdbu, 0x404858ebu, 0x404921fbu};

/* 2/pi: bits after the binary point, 32 per word (1280 bits). */
static const uint32_t TWO_OVER_PI[40] = {
  0xa2f9836eu, 0x4e441529u, 0xfc2757d1u, 0xf534ddc0u, 0xdb629599u, 0x3c439041u, 0xfe5163abu, 0xdebbc561u,
  0xb7246e3au, 0x424dd2e0u, 0x06492eeau, 0x09d1921cu, 0xfe1deb1cu, 0xb129a73eu, 0xe88235f5u, 0x2ebb4484u,
  0xe99c7026u, 0xb45f7e41u, 0x3991d639u, 0x835339f4u, 0x9c845f8bu, 0xbdf9283bu, 0x1ff897ffu, 0xde05980fu,
  0xef2f118bu, 0x5a0a6d1fu, 0x6d367ecfu, 0x27cb09b7u, 0x4f463f66u, 0x9e5fea2du, 0x7527bac7u, 0xebe5f17bu,
  0x3d0739f7u, 0x8a5292eau, 0x6bfb5fb1u, 0x1f8d5d08u, 0x56033046u, 0xfc7b6babu, 0xf0cfbc20u, 0x9af4361du};
/* floor(pi/2 * 2^126), little-endian 32-bit limbs. */
static const uint32_t PIO2_126[4] = {0xc06e0e68u, 0x62633145u, 0x10b4611au, 0x6487ed51u};

/* ------------------------------------------- exact Payne-Hanek reduction -- */
static inline int wbit(const uint32_t* p, int nw, int k)
{
  if (k < 0 || k >= 32 * nw) return 0;
  return (int)((p[k >> 5] >> (k & 31)) & 1u);
}
static uint64_t wbits64(const uint32_t* p, int nw, int k)   /* bits [k, k+64) */
{
  uint64_t r = 0;
  for (int i = 63; i >= 0; --i) r = (r << 1) | (uint64_t)wbit(p, nw, k + i);
  return r;
}
static int wany_below(const uint32_t* p, int nw, int k)      /* any bit in [0, k) */
{
  for (int i = 0; i < k && i < 32 * nw; ++i)
    if (wbit(p, nw, i)) return 1;
  return 0;
}

/* x = m * 2^q (m < 2^53, x > 0 finite).  n = round(x * 2/pi) mod 4 and
 * r = x - n*pi/2 rounded once to `prec` bits. */
static int exact_rem_pio2(uint64_t m, int q, int prec, double* r)
{
  enum { K = 7 };
  const int i0 = q >= 2 ? (q - 2) / 32 : 0;   /* earlier words only add multiples of 4 */
  uint32_t nw[K], p[K + 2];
  memset(p, 0, sizeof p);
  for (int b = 0; b < K; ++b) nw[b] = TWO_OVER_PI[i0 + K - 1 - b];
  const uint32_t ma[2] = {(uint32_t)m, (uint32_t)(m >> 32)};
  for (int a = 0; a < 2; ++a) {
    uint64_t c = 0;
    for (int b = 0; b < K; ++b) {
      uint64_t t = (uint64_t)ma[a] * nw[b] + p[a + b] + c;
      p[a + b] = (uint32_t)t;
      c = t >> 32;
    }
    p[a + K] = (uint32_t)c;
  }
  const int sh = 32 * (i0 + K) - q;           /* fraction bits of p */
  int n = wbit(p, K + 2, sh) | (wbit(p, K + 2, sh + 1) << 1);
  uint32_t f[K + 2];
  for (int k = 0; k < K + 2; ++k) {
    const int lo = 32 * k;
    f[k] = lo >= sh ? 0u : (lo + 32 > sh ? (p[k] & ((1u << (sh - lo)) - 1u)) : p[k]);
  }
  const int neg = wbit(f, K + 2, sh - 1);
  if (neg) {                                   /* f = 2^sh - f, n = n + 1 */
    n += 1;
    uint64_t c = 1;
    for (int k = 0; k < K + 2; ++k) {
      const int lo = 32 * k;
      const uint32_t mask = lo >= sh ? 0u : (lo + 32 > sh ? ((1u << (sh - lo)) - 1u) : 0xffffffffu);
      uint64_t t = (uint64_t)(~f[k] & mask) + c;
      f[k] = (uint32_t)t & mask;
      c = t >> 32;
    }
  }
  int top = -1;
  for (int k = 32 * (K + 2) - 1; k >= 0; --k)
    if (wbit(f, K + 2, k)) { top = k; break; }
  if (top < 0) { *r = 0.0; return n & 3; }
  uint32_t M[4];
  for (int j = 0; j < 4; ++j) M[j] = (uint32_t)wbits64(f, K + 2, top - 127 + 32 * j);
  const int sticky_f = wany_below(f, K + 2, top - 127);
  uint32_t Q[8];
  memset(Q, 0, sizeof Q);
  for (int a = 0; a < 4; ++a) {
    uint64_t c = 0;
    for (int b = 0; b < 4; ++b) {
      uint64_t t = (uint64_t)M[a] * PIO2_126[b] + Q[a + b] + c;
      Q[a + b] = (uint32_t)t;
      c = t >> 32;
    }
    Q[a + 4] = (uint32_t)c;
  }
  /* |r| = Q * 2^(top - 127 - sh - 126) */
  const int T = wbit(Q, 8, 254) ? 254 : 253;
  const uint64_t mant = wbits64(Q, 8, T - 63);
  const int sticky = sticky_f || wany_below(Q, 8, T - 63);
  const int drop = 64 - prec;
  uint64_t mm = mant >> drop;
  const uint64_t rem = mant & ((1ull << drop) - 1u), half = 1ull << (drop - 1);
  int e = (T - 63) + (top - 253 - sh) + drop;
  if (rem > half || (rem == half && (sticky || (mm & 1u)))) ++mm;
  if (mm >> prec) { mm >>= 1; ++e; }
  const double v = ldexp((double)mm, e);
  *r = neg ? -v : v;
  return n & 3;
}

/* ------------------------------------------------- float reductions ------ */
static inline float r2e_tf(float a) { return rintf(a); }
static inline double r2e_td(double a) { return rint(a); }
/* cvttps2dq / cvttpd2dq: out of range or NaN gives INT32_MIN */
static inline int32_t toint32(double a)
{
  return (a != a || a >= 2147483648.0 || a < -2147483648.0) ? INT32_MIN : (int32_t)a;
}
static inline int64_t toint64(double a)
{
  return (a != a || a >= 9223372036854775808.0 || a < -9223372036854775808.0) ? INT64_MIN : (int64_t)a;
}

static int straight_f(float x, float* xr)
{
  float r = x - tfb(F_PIO2_1);
  r -= tfb(F_PIO2_2);
  r -= tfb(F_PIO2_3);
  *xr = r;
  return 1;
}
static int cephes_f(float x, float* xr)
{
  const float xi = r2e_tf(x * tfb(F_TWOOPI));
  float r = x - xi * tfb(F_PIO2_1);
  r -= xi * tfb(F_PIO2_2);
  r -= xi * tfb(F_PIO2_3);
  *xr = r;
  return toint32(xi) & 3;
}
static int medium_f(float t, float* xr)
{
  const float fn = r2e_tf(t * tfb(F_INVPIO2));
  float r = t - fn * tfb(F_PIO2_1);
  float t2 = r, w = fn * tfb(F_PIO2_2);
  r = t2 - w;
  w = fn * tfb(F_PIO2_2T) - ((t2 - r) - w);
  t2 = r;
  w = fn * tfb(F_PIO2_3);
  r = t2 - w;
  w = fn * tfb(F_PIO2_3T) - ((t2 - r) - w);
  *xr = r - w;
  return toint32(fn) & 3;
}
/* fdlibm __ieee754_rem_pio2f for x >= 0 (scalar/rem_pio2.hpp:148-231) */
static int fdlibm_f(float x, float* xr)
{
  const uint32_t ix = tbf(x) & 0x7fffffffu;
  if (ix <= 0x3f490fd8u) { *xr = x; return 0; }
  if (ix < 0x4016cbe4u) {
    float z = x - tfb(F_PIO2_1);
    if ((ix & 0xfffffff0u) != 0x3fc90fd0u) *xr = z - tfb(F_PIO2_1T);
    else { z -= tfb(F_PIO2_2); *xr = z - tfb(F_PIO2_2T); }
    return 1;
  }
  if (ix <= 0x43490f80u) {
    const int32_t n = (int32_t)(x * tfb(F_INVPIO2) + 0.5f);
    const float fn = (float)n;
    float r = x - fn * tfb(F_PIO2_1), w = fn * tfb(F_PIO2_1T), y0;
    if (n < 32 && (ix & 0xffffff00u) != NPIO2_HW_F[n - 1]) {
      y0 = r - w;
    } else {
      const int j = (int)(ix >> 23);
      y0 = r - w;
      int i = j - (int)((tbf(y0) >> 23) & 0xffu);
      if (i > 8) {
        float t = r;
        w = fn * tfb(F_PIO2_2);
        r = t - w;
        w = fn * tfb(F_PIO2_2T) - ((t - r) - w);
        y0 = r - w;
        i = j - (int)((tbf(y0) >> 23) & 0xffu);
        if (i > 25) {
          t = r;
          w = fn * tfb(F_PIO2_3);
          r = t - w;
          w = fn * tfb(F_PIO2_3T) - ((t - r) - w);
          y0 = r - w;
        }
      }
    }
    *xr = y0;
    return n & 3;
  }
  if (ix >= 0x7f800000u) { *xr = x - x; return 0; }
  double r;
  const int n = exact_rem_pio2((uint64_t)((ix & 0x7fffffu) | 0x800000u), (int)(ix >> 23) - 150, 24, &r);
  *xr = (float)r;
  return n;
}

/* ------------------------------------------------ double reductions ------ */
static int straight_d(double x, double* xr)
{
  double r = x - tdb(D_PIO2_1);
  r -= tdb(D_PIO2_2);
  r -= tdb(D_PIO2_3);
  *xr = r;
  return 1;
}
static int cephes_d(double x, double* xr)
{
  const double xi = r2e_td(x * tdb(D_TWOOPI));
  double r = x - xi * tdb(D_PIO2_1);
  r -= xi * tdb(D_PIO2_2);
  r -= xi * tdb(D_PIO2_3);
  *xr = r;
  return (int)(toint64(xi) & 3);
}
static int medium_d(double t, double* xr)
{
  const double fn = r2e_td(t * tdb(D_INVPIO2));
  double r = t - fn * tdb(D_PIO2_1);
  double t2 = r, w = fn * tdb(D_PIO2_2);
  r = t2 - w;
  w = fn * tdb(D_PIO2_2T) - ((t2 - r) - w);
  t2 = r;
  w = fn * tdb(D_PIO2_3);
  r = t2 - w;
  w = fn * tdb(D_PIO2_3T) - ((t2 - r) - w);
  *xr = r - w;
  return (int)(toint64(fn) & 3);
}
/* NT2's double rem_pio2 (scalar/rem_pio2.hpp:413-427) over fdlibm
 * __ieee754_rem_pio2 for x >= 0 (:536-621) */
static int fdlibm_d(double x, double* xr)
{
  if (x == INFINITY) { *xr = NAN; return 0; }
  const uint32_t ix = (uint32_t)(tbd(x) >> 32) & 0x7fffffffu;
  if (ix <= 0x3fe921fbu) { *xr = x; return 0; }
  if (ix < 0x4002d97cu) {
    double z = x - tdb(D_PIO2_1);
    if (ix != 0x3ff921fbu) *xr = z - tdb(D_PIO2_1T);
    else { z -= tdb(D_PIO2_2); *xr = z - tdb(D_PIO2_2T); }
    return 1;
  }
  if (ix <= 0x413921fbu) {
    const int32_t n = (int32_t)(x * tdb(D_INVPIO2) + 0.5);
    const double fn = (double)n;
    double r = x - fn * tdb(D_PIO2_1), w = fn * tdb(D_PIO2_1T), y0;
    if (n < 32 && n > 0 && ix != NPIO2_HW_D[n - 1]) {
      y0 = r - w;
    } else {
      const int j = (int)(ix >> 20);
      y0 = r - w;
      int i = j - (int)((tbd(y0) >> 52) & 0x7ffu);
      if (i > 16) {
        double t = r;
        w = fn * tdb(D_PIO2_2);
        r = t - w;
        w = fn * tdb(D_PIO2_2T) - ((t - r) - w);
        y0 = r - w;
        i = j - (int)((tbd(y0) >> 52) & 0x7ffu);
        if (i > 49) {
          t = r;
          w = fn * tdb(D_PIO2_3);
          r = t - w;
          w = fn * tdb(D_PIO2_3T) - ((t - r) - w);
          y0 = r - w;
        }
      }
    }
    *xr = y0;
    return n & 3;
  }
  if (ix >= 0x7ff00000u) { *xr = x - x; return 0; }
  const uint64_t b = tbd(x);
  return exact_rem_pio2((b & 0xfffffffffffffull) | (1ull << 52), (int)((b >> 52) & 0x7ffu) - 1075, 53, xr);
}

/* Level of one lane (number of thresholds |x| exceeds; NaN is level 0). */
static inline int level_f(float x)
{
  return (x > tfb(F_PIO4)) + (x > tfb(F_PIO2)) + (x > tfb(F_20PI)) + (x > tfb(F_MEDPI)) + (x > tfb(F_DMPI));
}
static inline int level_d(double x)
{
  return (x > tdb(D_PIO4)) + (x > tdb(D_PIO2)) + (x > tdb(D_20PI)) + (x > tdb(D_MEDPI));
}

/* The double chain over lanes x[0..k) (one SIMD pack of doubles). */
static void reduce_pack_d(const double* x, int k, double* xr, int* n)
{
  int lv = 0;
  for (int l = 0; l < k; ++l) { const int v = level_d(x[l]); lv = v > lv ? v : lv; }
  for (int l = 0; l < k; ++l) {
    switch (lv) {
      case 0: xr[l] = x[l]; n[l] = 0; break;
      case 1: n[l] = straight_d(x[l], &xr[l]); break;
      case 2: n[l] = cephes_d(x[l], &xr[l]); break;
      case 3: n[l] = medium_d(x[l], &xr[l]); break;
      default: n[l] = fdlibm_d(x[l], &xr[l]); break;
    }
  }
}

/* The float chain over one pack of k lanes. */
static void reduce_pack_f(const float* x, int k, float* xr, int* n)
{
  int lv = 0;
  for (int l = 0; l < k; ++l) { const int v = level_f(x[l]); lv = v > lv ? v : lv; }
  if (lv == 4) {                     /* halves of the pack through the double chain */
    const int h = k > 1 ? k / 2 : 1;
    for (int s = 0; s < k; s += h) {
      double xd[8], rd[8];
      for (int l = 0; l < h; ++l) xd[l] = (double)x[s + l];
      reduce_pack_d(xd, h, rd, n + s);
      for (int l = 0; l < h; ++l) xr[s + l] = (float)rd[l];
    }
    return;
  }
  for (int l = 0; l < k; ++l) {
    switch (lv) {
      case 0: xr[l] = x[l]; n[l] = 0; break;
      case 1: n[l] = straight_f(x[l], &xr[l]); break;
      case 2: n[l] = cephes_f(x[l], &xr[l]); break;
      case 3: n[l] = medium_f(x[l], &xr[l]); break;
      default: n[l] = fdlibm_f(x[l], &xr[l]); break;
    }
  }
}

/* --------------------------------------------------------- evaluation ---- */
/* simd/common/impl/trigo/f_trig_evaluation.hpp:25-56 */
static inline float hornerf(float x, const uint32_t* c, int k)
{
  float a = tfb(c[0]);
  for (int i = 1; i < k; ++i) a = x * a + tfb(c[i]);
  return a;
}
static inline double hornerd(double x, const uint64_t* c, int k)
{
  double a = tdb(c[0]);
  for (int i = 1; i < k; ++i) a = x * a + tdb(c[i]);
  return a;
}
static const uint32_t COS_F[3] = {0x37ccf5ceu, 0xbab60619u, 0x3d2aaaa5u};
static const uint32_t SIN_F[3] = {0xb94ca1f9u, 0x3c08839du, 0xbe2aaaa2u};
static const uint32_t TAN_F[6] = {0x3c19c53bu, 0x3b4c779cu, 0x3cc821b5u, 0x3d5ac5c9u, 0x3e0896ddu, 0x3eaaaa6fu};
static const uint64_t COS_D[7] = {0x3da8ff831ad9b219ull, 0xbe21eea7c1e514d4ull, 0x3e927e4f8e06d9a5ull,
                                  0xbefa01a019ddbcd9ull, 0x3f56c16c16c15d47ull, 0xbfa5555555555551ull,
                                  0x3fe0000000000000ull};
static const uint64_t SIN_D[6] = {0x3de5d8fd1fcf0ec1ull, 0xbe5ae5e5a9291691ull, 0x3ec71de3567d4896ull,
                                  0xbf2a01a019bfdf03ull, 0x3f8111111110f7d0ull, 0xbfc5555555555548ull};
static const uint64_t TAN_DN[3] = {0xc0c992d8d24f3f38ull, 0x413199eca5fc9dddull, 0xc1711fead3299176ull};
static const uint64_t TAN_DD[5] = {0x3ff0000000000000ull, 0x40cab8a5eeb36572ull, 0xc13427bc582abc96ull,
                                   0x4177d98fc2ead8efull, 0xc189afe03cbe5a31ull};

static inline float cos_eval_f(float z)
{
  const float y = hornerf(z, COS_F, 3);
  return 1.0f + (z * -0.5f + y * (z * z));
}
static inline float sin_eval_f(float z, float x) { return (hornerf(z, SIN_F, 3) * z) * x + x; }
static inline float tan_eval_f(float x)
{
  const float zz = x * x;
  return (hornerf(zz, TAN_F, 6) * zz) * x + x;
}
static inline double cos_eval_d(double z) { return 1.0 - hornerd(z, COS_D, 7) * z; }
static inline double sin_eval_d(double z, double x) { return (hornerd(z, SIN_D, 6) * z) * x + x; }
static inline double tan_eval_d(double x)
{
  const double zz = x * x;
  return x + x * (zz * (hornerd(zz, TAN_DN, 3) / hornerd(zz, TAN_DD, 5)));
}

enum { TRIG_SIN = 0, TRIG_COS = 1, TRIG_TAN = 2, TRIG_SINPI = 3, TRIG_COSPI = 4,
       TRIG_ASIN = 5, TRIG_ACOS = 6, TRIG_ATAN = 7,
       TRIG_COT = 8, TRIG_TANPI = 9, TRIG_COTPI = 10, TRIG_SIND = 11, TRIG_COSD = 12, TRIG_TAND = 13,
       TRIG_COTD = 14 };
/* which reduction a kind takes: radian (pack-level method), pi_tag or degree_tag */
static inline int is_pi_kind(int k) { return k == TRIG_SINPI || k == TRIG_COSPI || k == TRIG_TANPI || k == TRIG_COTPI; }
static inline int is_deg_kind(int k) { return k >= TRIG_SIND && k <= TRIG_COTD; }

/* ------------------------------------------------ inverse functions ----- */
/* NT2's SIMD forms (functions/simd/common/impl/invtrig/{f,d}_invtrig.hpp), element by element
 * (no pack dependence).  seladd/ifadd/ifnotadd are unconditional adds of a selected value
 * (boost/simd/boolean/functions/simd/common/{seladd,ifnotadd}.hpp); fms(a,b,c) = a*b - c
 * (boost/simd/arithmetic/functions/generic/fms.hpp).  NT2's scalar forms differ (float acos,
 * double asin/acos/atan; functions/scalar/impl/invtrig/{f,d}_invtrig.hpp): not restated. */
#define F_PIO2LO 0xb33bbd2eu
#define F_PIO4LO 0xb2bbbd2eu
#define F_TAN3PIO8 0x401a827au
#define F_TANPIO8 0x3ed413cdu
#define D_PIO2LO 0x3c91a62633145c07ull
#define D_PIO4LO 0x3c81a62633145c07ull
#define D_TAN3PIO8 0x4003504f333f9de6ull
#define D_TANPIO8 0x3fda827999fcef31ull
#define D_SQRTEPS 0x3e50000000000000ull

static const uint32_t ASIN_F[5] = {0x3d2cb352u, 0x3cc617e3u, 0x3d3a3ec7u, 0x3d9980f6u, 0x3e2aaae4u};
static const uint32_t ATAN_F[4] = {0x3da4f0d1u, 0xbe0e1b85u, 0x3e4c925fu, 0xbeaaaa2au};
static const uint64_t ASIN_D_P1[5] = {0x3f684fc3988e9f08ull, 0xbfe2079259f9290full, 0x401bdff5baf33e6aull,
                                      0xc03991aaac01ab68ull, 0x403c896240f3081dull};
static const uint64_t ASIN_D_Q1[5] = {0x3ff0000000000000ull, 0xc035f2a2b6bf5d8cull, 0x40626219af6a7f42ull,
                                      0xc077fe08959063eeull, 0x40756709b0b644beull};
static const uint64_t ASIN_D_P2[6] = {0x3f716b9b0bd48ad3ull, 0xbfe34341333e5c16ull, 0x4015c74b178a2dd9ull,
                                      0xc0304331de27907bull, 0x40339007da779259ull, 0xc020656c06ceafd5ull};
static const uint64_t ASIN_D_Q2[6] = {0x3ff0000000000000ull, 0xc02d7b590b5e0eabull, 0x40519fc025fe9054ull,
                                      0xc06265bb6d3576d7ull, 0x4061705684ffbf9dull, 0xc04898220a3607acull};
static const uint64_t ATAN_D_P[5] = {0xbfec007fa1f72594ull, 0xc03028545b6b807aull, 0xc052c08c36880273ull,
                                     0xc05eb8bf2d05ba25ull, 0xc0503669fd28ec8eull};
static const uint64_t ATAN_D_Q[6] = {0x3ff0000000000000ull, 0x4038dbc45b14603cull, 0x4064a0dd43b8fa25ull,
                                     0x407b0e18d2e2be3bull, 0x407e563f13b049eaull, 0x4068519efbbd62ecull};

/* f_invtrig.hpp:31-57 */
static float asin_f(float a0)
{
  float x = fabsf(a0);
  const uint32_t sign = tbf(a0) & 0x80000000u;
  const int larger = x > 0.5f;
  float z = larger ? 0.5f * (1.0f - x) : x * x;
  x = larger ? sqrtf(z) : x;
  float z1 = hornerf(z, ASIN_F, 5);
  z1 = z1 * (z * x) + x;
  z = larger ? tfb(F_PIO2) - (z1 + z1) : z1;
  return tfb(tbf(z) ^ sign);
}
/* f_invtrig.hpp:58-71 */
static float acos_f(float a0)
{
  float x = fabsf(a0);
  const int larger = x > 0.5f;
  x = larger ? sqrtf(-0.5f * x + 0.5f) : a0;
  x = asin_f(x);
  x = x + (larger ? x : 0.0f);
  x = (a0 < -0.5f) ? tfb(F_PI) - x : x;
  return larger ? x : tfb(F_PIO2) - x;
}
/* f_invtrig.hpp:78-110: atan(|a0|) */
static float kernel_atan_f(float a0)
{
  const float x = fabsf(a0);
  const int flag1 = x < tfb(F_TAN3PIO8);
  const int flag2 = x >= tfb(F_TANPIO8) && flag1;
  float yy = flag1 ? 0.0f : tfb(F_PIO2);
  yy = flag2 ? tfb(F_PIO4) : yy;
  float xx = flag1 ? x : -(1.0f / x);
  xx = flag2 ? (x - 1.0f) / (x + 1.0f) : xx;
  const float z = xx * xx;
  float z1 = hornerf(z, ATAN_F, 4);
  z1 = xx * (z1 * z) + xx;
  z1 = z1 + (flag2 ? tfb(F_PIO4LO) : 0.0f);
  z1 = z1 + (flag1 ? 0.0f : tfb(F_PIO2LO));
  return yy + z1;
}
/* f_invtrig.hpp:72-77 */
static float atan_f(float a0) { return tfb(tbf(kernel_atan_f(a0)) ^ (tbf(a0) & 0x80000000u)); }
/* d_invtrig.hpp:29-86 */
static double asin_d(double a0)
{
  const double x = fabs(a0);
  const int small = x < tdb(D_SQRTEPS);
  double zz1 = 1.0 - x;
  const double vp = zz1 * hornerd(zz1, ASIN_D_P1, 5) / hornerd(zz1, ASIN_D_Q1, 5);
  zz1 = sqrt(zz1 + zz1);
  double z = tdb(D_PIO4) - zz1;
  zz1 = zz1 * vp - tdb(D_PIO2LO);
  z = z - zz1;
  zz1 = z + tdb(D_PIO4);
  double zz2 = a0 * a0;
  z = zz2 * hornerd(zz2, ASIN_D_P2, 6) / hornerd(zz2, ASIN_D_Q2, 6);
  zz2 = x * z + x;
  if (x > 1.0) return NAN;
  const double r = small ? x : (x > 0.625 ? zz1 : zz2);
  return tdb(tbd(r) ^ (tbd(a0) & 0x8000000000000000ull));
}
/* d_invtrig.hpp:87-97 */
static double acos_d(double a0)
{
  double x = fabs(a0);
  const int larger = x > 0.5;
  x = larger ? sqrt(-0.5 * x + 0.5) : a0;
  x = asin_d(x);
  x = x + (larger ? x : 0.0);
  x = (a0 < -0.5) ? tdb(D_PI) - x : x;
  return larger ? x : tdb(D_PIO2) - x;
}
/* d_invtrig.hpp:104-139: atan(|a0|) */
static double kernel_atan_d(double a0)
{
  const double x = fabs(a0);
  const int flag1 = x < tdb(D_TAN3PIO8);
  const int flag2 = x >= tdb(D_TANPIO8) && flag1;
  double yy = flag1 ? 0.0 : tdb(D_PIO2);
  yy = flag2 ? tdb(D_PIO4) : yy;
  double xx = flag1 ? x : -(1.0 / x);
  xx = flag2 ? (x - 1.0) / (x + 1.0) : xx;
  double z = xx * xx;
  z = z * hornerd(z, ATAN_D_P, 5) / hornerd(z, ATAN_D_Q, 6);
  z = xx * z + xx;
  z = z + (flag2 ? tdb(D_PIO4LO) : 0.0);
  z = z + (flag1 ? 0.0 : tdb(D_PIO2LO));
  return yy + z;
}
/* d_invtrig.hpp:98-103 */
static double atan_d(double a0) { return tdb(tbd(kernel_atan_d(a0)) ^ (tbd(a0) & 0x8000000000000000ull)); }

/* atan2(a0, a1), NT2's SIMD form (functions/simd/common/atan2.hpp:31-52): both infinite
 * -> +-1 each; kernel_atan(a0/a1); Pi minus it unless a1 > 0; the sign of a0 (negatenz,
 * -0 counts as negative); a0 == 0 -> (a1 < 0 ? Pi : 0); NaN if either is NaN. */
static float atan2_f(float a0, float a1)
{
  if (isinf(a0) && isinf(a1)) { a0 = copysignf(1.0f, a0); a1 = copysignf(1.0f, a1); }
  float z = kernel_atan_f(a0 / a1);
  z = (a1 > 0.0f) ? z : tfb(F_PI) - z;
  z = (tbf(a0) & 0x80000000u) ? -z : z;
  z = (a0 == 0.0f) ? ((a1 < 0.0f) ? tfb(F_PI) : 0.0f) : z;
  return (isnan(a0) || isnan(a1)) ? NAN : z;
}
static double atan2_d(double a0, double a1)
{
  if (isinf(a0) && isinf(a1)) { a0 = copysign(1.0, a0); a1 = copysign(1.0, a1); }
  double z = kernel_atan_d(a0 / a1);
  z = (a1 > 0.0) ? z : tdb(D_PI) - z;
  z = (tbd(a0) & 0x8000000000000000ull) ? -z : z;
  z = (a0 == 0.0) ? ((a1 < 0.0) ? tdb(D_PI) : 0.0) : z;
  return (isnan(a0) || isnan(a1)) ? NAN : z;
}
EXPORT void nt2o_atan2_f(const float* a0, const float* a1, float* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) y[i] = atan2_f(a0[i], a1[i]);
}
EXPORT void nt2o_atan2_d(const double* a0, const double* a1, double* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) y[i] = atan2_d(a0[i], a1[i]);
}
static inline float inv_f(int kind, float a)
{
  return kind == TRIG_ASIN ? asin_f(a) : (kind == TRIG_ACOS ? acos_f(a) : atan_f(a));
}
static inline double inv_d(int kind, double a)
{
  return kind == TRIG_ASIN ? asin_d(a) : (kind == TRIG_ACOS ? acos_d(a) : atan_d(a));
}

/* NT2's invalid-argument tests of tana / cota per unit (scalar/impl/trigo/trig_reduction.hpp:89-90,
 * 268-269, 308-309): none in radians; pi_tag: tan at x - 1/2 integral, cot at nonzero integers;
 * degree_tag: tan at (x - 90)/180 integral, cot at nonzero x/180 integral. */
static int flint_f(float x);
static inline int tan_invalid_f(int kind, float a0)
{
  if (kind == TRIG_TANPI) return flint_f(a0 - 0.5f);
  if (kind == TRIG_TAND) return flint_f((a0 - 90) * tfb(0x3bb60b61u));
  return 0;
}
static inline int cot_invalid_f(int kind, float a0)
{
  if (kind == TRIG_COTPI) return a0 != 0 && flint_f(a0);
  if (kind == TRIG_COTD) return a0 != 0 && flint_f(a0 * tfb(0x3bb60b61u));
  return 0;
}
/* trig_base sina / cosa / tana / cota (simd/common/impl/trigo/trig_base.hpp:72-141) */
static inline float finish_f(int kind, float a0, float xr, int n)
{
  const uint32_t sgn = tbf(a0) & (uint32_t)1 << 31;
  if (kind == TRIG_TAN || kind == TRIG_TANPI || kind == TRIG_TAND) {
    float y = tan_eval_f(xr);
    if (n & 1) y = -(1.0f / y);
    y = tfb(tbf(y) ^ sgn);
    return tan_invalid_f(kind, a0) ? (float)NAN : y;
  }
  if (kind == TRIG_COT || kind == TRIG_COTPI || kind == TRIG_COTD) {
    float y = tan_eval_f(xr);
    y = (n & 1) ? -y : 1.0f / y;
    y = tfb(tbf(y) ^ sgn);
    y = cot_invalid_f(kind, a0) ? (float)NAN : y;
    return a0 != 0 ? y : 1.0f / a0;
  }
  const float z = xr * xr;
  const int swap = n & 1;
  if (kind == TRIG_SIN || kind == TRIG_SINPI || kind == TRIG_SIND) {
    const float v = swap ? cos_eval_f(z) : sin_eval_f(z, xr);
    return tfb(tbf(v) ^ sgn ^ ((uint32_t)(n & 2) << (31 - 1)));
  }
  const float v = swap ? sin_eval_f(z, xr) : cos_eval_f(z);
  return tfb(tbf(v) ^ ((uint32_t)((n ^ (n >> 1)) & 1) << 31));
}
/* NT2's invalid-argument tests of tana / cota per unit (scalar/impl/trigo/trig_reduction.hpp:89-90,
 * 268-269, 308-309): none in radians; pi_tag: tan at x - 1/2 integral, cot at nonzero integers;
 * degree_tag: tan at (x - 90)/180 integral, cot at nonzero x/180 integral. */
static int flint_d(double x);
static inline int tan_invalid_d(int kind, double a0)
{
  if (kind == TRIG_TANPI) return flint_d(a0 - 0.5);
  if (kind == TRIG_TAND) return flint_d((a0 - 90) * tdb(0x3f76c16c16c16c17ull));
  return 0;
}
static inline int cot_invalid_d(int kind, double a0)
{
  if (kind == TRIG_COTPI) return a0 != 0 && flint_d(a0);
  if (kind == TRIG_COTD) return a0 != 0 && flint_d(a0 * tdb(0x3f76c16c16c16c17ull));
  return 0;
}
/* trig_base sina / cosa / tana / cota (simd/common/impl/trigo/trig_base.hpp:72-141) */
static inline double finish_d(int kind, double a0, double xr, int n)
{
  const uint64_t sgn = tbd(a0) & (uint64_t)1 << 63;
  if (kind == TRIG_TAN || kind == TRIG_TANPI || kind == TRIG_TAND) {
    double y = tan_eval_d(xr);
    if (n & 1) y = -(1.0 / y);
    y = tdb(tbd(y) ^ sgn);
    return tan_invalid_d(kind, a0) ? (double)NAN : y;
  }
  if (kind == TRIG_COT || kind == TRIG_COTPI || kind == TRIG_COTD) {
    double y = tan_eval_d(xr);
    y = (n & 1) ? -y : 1.0 / y;
    y = tdb(tbd(y) ^ sgn);
    y = cot_invalid_d(kind, a0) ? (double)NAN : y;
    return a0 != 0 ? y : 1.0 / a0;
  }
  const double z = xr * xr;
  const int swap = n & 1;
  if (kind == TRIG_SIN || kind == TRIG_SINPI || kind == TRIG_SIND) {
    const double v = swap ? cos_eval_d(z) : sin_eval_d(z, xr);
    return tdb(tbd(v) ^ sgn ^ ((uint64_t)(n & 2) << (63 - 1)));
  }
  const double v = swap ? sin_eval_d(z, xr) : cos_eval_d(z);
  return tdb(tbd(v) ^ ((uint64_t)((n ^ (n >> 1)) & 1) << 63));
}

/* pi_tag reduction (trig_reduction.hpp:216-229): xi = round2even(2x),
 * xr = (x - xi/2) * pi, n = fast_toint(xi). */
static inline int reduce_pi_f(float x, float* xr)
{
  const float xi = r2e_tf(x * 2.0f);
  *xr = (x - xi * 0.5f) * tfb(F_PI);
  return toint32(xi) & 3;
}
static inline int reduce_pi_d(double x, double* xr, int simd)
{
  const double xi = r2e_td(x * 2.0);
  *xr = (x - xi * 0.5) * tdb(D_PI);
  /* SSE2 converts packed doubles through int32 (cvttpd2dq); scalar code casts to int64 */
  return simd ? (toint32(xi) & 3) : (int)(toint64(xi) & 3);
}
/* degree_tag reduction (trig_reduction.hpp:262-278, the form without x87): xi = round2even(x/90),
 * xr = inrad(x - xi*90), n = fast_toint(xi) (through int32 for packed doubles, as for pi_tag). */
static inline int reduce_deg_f(float x, float* xr)
{
  const float xi = r2e_tf(x * tfb(0x3c360b61u));
  *xr = (x - xi * 90.0f) * tfb(0x3c8efa35u);
  return toint32(xi) & 3;
}
static inline int reduce_deg_d(double x, double* xr, int simd)
{
  const double xi = r2e_td(x * tdb(0x3f86c16c16c16c17ull));
  *xr = (x - xi * 90.0) * tdb(0x3f91df46a2529d39ull);
  return simd ? (toint32(xi) & 3) : (int)(toint64(xi) & 3);
}

static void trig_pack_f(int kind, const float* a, float* y, int k)
{
  float x[8], xr[8];
  int n[8];
  for (int l = 0; l < k; ++l) x[l] = fabsf(a[l]);
  if (is_pi_kind(kind)) {
    for (int l = 0; l < k; ++l) n[l] = reduce_pi_f(x[l], &xr[l]);
  } else if (is_deg_kind(kind)) {
    for (int l = 0; l < k; ++l) n[l] = reduce_deg_f(x[l], &xr[l]);
  } else {
    reduce_pack_f(x, k, xr, n);
  }
  for (int l = 0; l < k; ++l) y[l] = finish_f(kind, a[l], xr[l], n[l]);
}
static void trig_pack_d(int kind, const double* a, double* y, int k)
{
  double x[8], xr[8];
  int n[8];
  for (int l = 0; l < k; ++l) x[l] = fabs(a[l]);
  if (is_pi_kind(kind)) {
    for (int l = 0; l < k; ++l) n[l] = reduce_pi_d(x[l], &xr[l], k > 1);
  } else if (is_deg_kind(kind)) {
    for (int l = 0; l < k; ++l) n[l] = reduce_deg_d(x[l], &xr[l], k > 1);
  } else {
    reduce_pack_d(x, k, xr, n);
  }
  for (int l = 0; l < k; ++l) y[l] = finish_d(kind, a[l], xr[l], n[l]);
}

/* y[i] = f(x[i]) over [0, n): packs of `pack` lanes from index 0, then the
 * n % pack tail one element at a time (NT2's scalar code). */
EXPORT int nt2o_trig_f(int kind, const float* x, float* y, size_t n, int pack)
{
  if (kind < 0 || kind > TRIG_COTD || pack < 1 || pack > 8) return 1;
  if (kind >= TRIG_ASIN && kind <= TRIG_ATAN) {
    for (size_t i = 0; i < n; ++i) y[i] = inv_f(kind, x[i]);
    return 0;
  }
  size_t i = 0;
  for (; i + (size_t)pack <= n; i += (size_t)pack) trig_pack_f(kind, x + i, y + i, pack);
  for (; i < n; ++i) trig_pack_f(kind, x + i, y + i, 1);
  return 0;
}
EXPORT int nt2o_trig_d(int kind, const double* x, double* y, size_t n, int pack)
{
  if (kind < 0 || kind > TRIG_COTD || pack < 1 || pack > 8) return 1;
  if (kind >= TRIG_ASIN && kind <= TRIG_ATAN) {
    for (size_t i = 0; i < n; ++i) y[i] = inv_d(kind, x[i]);
    return 0;
  }
  size_t i = 0;
  for (; i + (size_t)pack <= n; i += (size_t)pack) trig_pack_d(kind, x + i, y + i, pack);
  for (; i < n; ++i) trig_pack_d(kind, x + i, y + i, 1);
  return 0;
}

/* The reduction alone, for checking it: returns n, writes xr. */
EXPORT int nt2o_rem_pio2_exact_d(double x, double* xr)
{
  const uint64_t b = tbd(x);
  return exact_rem_pio2((b & 0xfffffffffffffull) | (1ull << 52), (int)((b >> 52) & 0x7ffu) - 1075, 53, xr);
}
EXPORT int nt2o_rem_pio2_exact_f(float x, float* xr)
{
  double r;
  const uint32_t b = tbf(x);
  const int n = exact_rem_pio2((uint64_t)((b & 0x7fffffu) | 0x800000u), (int)((b >> 23) & 0xffu) - 150, 24, &r);
  *xr = (float)r;
  return n;
}

/* -------------------------------------------------- fast forms ------ */
/* fast_sin ... fast_cotd (generic/fast_<name>.hpp): trig_base with the clipped_pio4_ mode, whose
 * style is "fast" (simd/common/impl/trigo/trig_base.hpp:67-135, scale at 143-149): no reduction;
 * x = (|x| > max_range ? NaN : x) * scale with (max_range, scale) = (pi/4, 1), (1/4, pi),
 * (45, pi/180) per unit; then sin_eval, cos_eval, base_tancot_eval or its reciprocal.
 * kind 0 sin 1 cos 2 tan 3 cot; unit 0 radian 1 pi 2 degree. */
static float fast_f(int kind, int unit, float a0)
{
  const float r = unit == 0 ? tfb(0x3f490fdbu) : (unit == 1 ? 0.25f : 45.0f);
  float x = fabsf(a0) > r ? NAN : a0;
  if (unit) x = x * (unit == 1 ? tfb(F_PI) : tfb(0x3c8efa35u));
  if (kind == 0) return sin_eval_f(x * x, x);
  if (kind == 1) return cos_eval_f(x * x);
  return kind == 2 ? tan_eval_f(x) : 1.0f / tan_eval_f(x);
}
static double fast_d(int kind, int unit, double a0)
{
  const double r = unit == 0 ? tdb(0x3fe921fb54442d18ull) : (unit == 1 ? 0.25 : 45.0);
  double x = fabs(a0) > r ? NAN : a0;
  if (unit) x = x * (unit == 1 ? tdb(D_PI) : tdb(0x3f91df46a2529d3aull));
  if (kind == 0) return sin_eval_d(x * x, x);
  if (kind == 1) return cos_eval_d(x * x);
  return kind == 2 ? tan_eval_d(x) : 1.0 / tan_eval_d(x);
}
/* proper_tanpi (simd/common/proper_tanpi.hpp:33-43): fast_tanpi of |x| or of 1/2 - |x|, the
 * sign of x, the reciprocal in the second case, NaN unless |x| <= 1/2. */
static float proper_tanpi_f(float a0)
{
  const float ax = fabsf(a0);
  const int test = ax <= 0.25f;
  float t = fast_f(2, 1, test ? ax : 0.5f - ax);
  t = a0 < 0.0f ? -t : t;
  return !(ax <= 0.5f) ? NAN : (test ? t : 1.0f / t);
}
static double proper_tanpi_d(double a0)
{
  const double ax = fabs(a0);
  const int test = ax <= 0.25;
  double t = fast_d(2, 1, test ? ax : 0.5 - ax);
  t = a0 < 0.0 ? -t : t;
  return !(ax <= 0.5) ? NAN : (test ? t : 1.0 / t);
}
/* nbd_atan2 (simd/common/nbd_atan2.hpp:35-42): atan2 without the infinity and NaN cases;
 * atan2d = indeg(atan2) (generic/atan2d.hpp). op 0 atan2d, 1 nbd_atan2. */
static float nbd_atan2_f(float a0, float a1)
{
  float z = kernel_atan_f(a0 / a1);
  z = (a1 > 0.0f) ? z : tfb(F_PI) - z;
  z = (tbf(a0) & 0x80000000u) ? -z : z;
  return (a0 == 0.0f) ? ((a1 < 0.0f) ? tfb(F_PI) : 0.0f) : z;
}
static double nbd_atan2_d(double a0, double a1)
{
  double z = kernel_atan_d(a0 / a1);
  z = (a1 > 0.0) ? z : tdb(D_PI) - z;
  z = (tbd(a0) & 0x8000000000000000ull) ? -z : z;
  return (a0 == 0.0) ? ((a1 < 0.0) ? tdb(D_PI) : 0.0) : z;
}
EXPORT void nt2o_atan2x_f(int op, const float* a0, const float* a1, float* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) {
    if (op == 1) { y[i] = nbd_atan2_f(a0[i], a1[i]); continue; }
    const float t = atan2_f(a0[i], a1[i]);
    y[i] = t * tfb(0x42652ee1u) - t * tfb(0xb53387c1u);
  }
}
EXPORT void nt2o_atan2x_d(int op, const double* a0, const double* a1, double* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) {
    if (op == 1) { y[i] = nbd_atan2_d(a0[i], a1[i]); continue; }
    const double t = atan2_d(a0[i], a1[i]);
    y[i] = t * tdb(0x404ca5dc1a63c1f8ull) - t * tdb(0xbce1e7ab456405f8ull);
  }
}

/* ------------------------------------------------- compositions ------ */
/* The trigonometric functors NT2 defines on top of the ones above
 * (modules/core/trigonometric/include/nt2/trigonometric/functions/generic headers and
 * simd/common/asec.hpp), op by op:
 *   0 csc = rec(sin)          1 sec = rec(cos)
 *   2 cscpi = NaN where x is a nonzero integer, else rec(sinpi)
 *   3 secpi = NaN where 2x is odd, else rec(cospi)
 *   4 cscd = cscpi(Oneo_180 * x)
 *   5 indeg = x*Radindeg - x*Radindegr      6 inrad = x*Deginrad
 *   7 acot = atan(rec)   8-10 asind, acosd, atand = indeg(asin, acos, atan)
 *   11-13 asinpi, acospi, atanpi = Invpi * (asin, acos, atan)
 *   14 acsc = asin(rec)  15 acscd = indeg(acsc)  16 asec = Pio_2 - acsc  17 asecd = indeg(asec)
 *   18 secd = rec(cosd), NaN where cosd is 0
 *   19-30 fast_sin, fast_cos, fast_tan, fast_cot, then the pi and the degree forms (fast_f)
 *   31 sinc = sin(x)/x, 32 sincpi = Invpi * (sinpi(x)/x): 1 for |x| < Eps, 0 for infinite x
 *      (simd/common/sinc.hpp:33-45, sincpi.hpp:33-45)
 *   33 proper_tanpi
 * rec is the IEEE quotient 1/x; the sin/cos based ones use the pack form of the
 * functors above (`pack` lanes). */
static int flint_f(float x) { return isfinite(x) && (x - truncf(x)) == 0.0f; }
static int flint_d(double x) { return isfinite(x) && (x - trunc(x)) == 0.0; }
#define TRIGX_BODY(T, SFX, FLINT, RADINDEG, RADINDEGR, DEGINRAD, INVPI, ONEO_180, PIO_2, FABS, EPS)     \
  if (op < 0 || op > 33) return 1;                                                                      \
  T* t = (T*)malloc((n ? n : 1) * sizeof(T));                                                          \
  if (!t) return 1;                                                                                     \
  int st = 0;                                                                                           \
  switch (op) {                                                                                         \
    case 0: case 1:                                                                                     \
      st = nt2o_trig_##SFX(op == 0 ? TRIG_SIN : TRIG_COS, x, y, n, pack);                              \
      for (size_t i = 0; i < n; ++i) y[i] = (T)1 / y[i];                                                \
      break;                                                                                            \
    case 2: case 4:                                                                                     \
      for (size_t i = 0; i < n; ++i) t[i] = op == 4 ? ONEO_180 * x[i] : x[i];                           \
      st = nt2o_trig_##SFX(TRIG_SINPI, t, y, n, pack);                                                  \
      for (size_t i = 0; i < n; ++i) y[i] = (FLINT(t[i]) && t[i] != 0) ? (T)NAN : (T)1 / y[i];         \
      break;                                                                                            \
    case 3:                                                                                             \
      st = nt2o_trig_##SFX(TRIG_COSPI, x, y, n, pack);                                                  \
      for (size_t i = 0; i < n; ++i) y[i] = FLINT(((x[i] * 2) - 1) * (T)0.5) ? (T)NAN : (T)1 / y[i];   \
      break;                                                                                            \
    case 33: for (size_t i = 0; i < n; ++i) y[i] = proper_tanpi_##SFX(x[i]); break;                   \
    case 31: case 32:                                                                                   \
      st = nt2o_trig_##SFX(op == 31 ? TRIG_SIN : TRIG_SINPI, x, y, n, pack);                            \
      for (size_t i = 0; i < n; ++i) {                                                                  \
        T r = y[i] / x[i];                                                                              \
        if (op == 32) r = INVPI * r;                                                                    \
        r = FABS(x[i]) < EPS ? (T)1 : r;                                                                \
        y[i] = isinf(x[i]) ? (T)0 : r;                                                                  \
      }                                                                                                 \
      break;                                                                                            \
    case 18:                                                                                            \
      st = nt2o_trig_##SFX(TRIG_COSD, x, y, n, pack);                                                   \
      for (size_t i = 0; i < n; ++i) y[i] = y[i] == 0 ? (T)NAN : (T)1 / y[i];                           \
      break;                                                                                            \
    case 19: case 20: case 21: case 22: case 23: case 24: case 25: case 26: case 27: case 28: case 29: case 30: \
      for (size_t i = 0; i < n; ++i) y[i] = fast_##SFX((op - 19) % 4, (op - 19) / 4, x[i]);              \
      break;                                                                                            \
    case 5: for (size_t i = 0; i < n; ++i) y[i] = x[i] * RADINDEG - x[i] * RADINDEGR; break;           \
    case 6: for (size_t i = 0; i < n; ++i) y[i] = x[i] * DEGINRAD; break;                               \
    case 7:                                                                                             \
      for (size_t i = 0; i < n; ++i) t[i] = (T)1 / x[i];                                                \
      st = nt2o_trig_##SFX(TRIG_ATAN, t, y, n, 1);                                                      \
      break;                                                                                            \
    default: {                                                                                          \
      const int inner = (op == 9 || op == 12) ? TRIG_ACOS : ((op == 10 || op == 13) ? TRIG_ATAN : TRIG_ASIN); \
      const int rec_first = op >= 14;                                                                   \
      for (size_t i = 0; i < n; ++i) t[i] = rec_first ? (T)1 / x[i] : x[i];                             \
      st = nt2o_trig_##SFX(inner, t, y, n, 1);                                                          \
      for (size_t i = 0; i < n; ++i) {                                                                  \
        T v = y[i];                                                                                     \
        if (op >= 11 && op <= 13) v = INVPI * v;                                                        \
        if (op == 16 || op == 17) v = PIO_2 - v;                                                        \
        if ((op >= 8 && op <= 10) || op == 15 || op == 17) v = v * RADINDEG - v * RADINDEGR;          \
        y[i] = v;                                                                                       \
      }                                                                                                 \
    }                                                                                                   \
  }                                                                                                     \
  free(t);                                                                                              \
  return st;
EXPORT int nt2o_trigx_f(int op, const float* x, float* y, size_t n, int pack)
{
  TRIGX_BODY(float, f, flint_f, tfb(0x42652ee1u), tfb(0xb53387c1u), tfb(0x3c8efa35u), tfb(0x3ea2f983u),
             tfb(0x3bb60b61u), tfb(0x3fc90fdbu), fabsf, tfb(0x34000000u))
}
EXPORT int nt2o_trigx_d(int op, const double* x, double* y, size_t n, int pack)
{
  TRIGX_BODY(double, d, flint_d, tdb(0x404ca5dc1a63c1f8ull), tdb(0xbce1e7ab456405f8ull), tdb(0x3f91df46a2529d39ull),
             tdb(0x3fd45f306dc9c883ull), tdb(0x3f76c16c16c16c17ull), tdb(0x3ff921fb54442d18ull), fabs,
             tdb(0x3cb0000000000000ull))
}
#undef TRIGX_BODY
