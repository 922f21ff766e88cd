/*
 * nt2_oracle.c -- CPU restatement of NT2's table-expression hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * evaluator in nt2_gb300/ and the timed CPU baseline of bench.py.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU legs load it; the
 * product path never calls it and has no CPU fallback.
 *
 * What it restates (paths relative to the NT2 source tree):
 *   - the Boost.SIMD / NT2 math functors used by the saxpy, sdot,
 *     Black-Scholes, rgb2grey, rgb2yuv, mandelbrot and sigmadelta expressions, in the form that
 *     NT2's SIMD transform body evaluates (the simd/common/... files), with
 *     the generic unfused fma/fnms (a*b+c rounded twice,
 *     modules/boost/simd/base/include/boost/simd/arithmetic/functions/generic/fma.hpp:32,
 *     generic/fnms.hpp:32);
 *   - the elementwise transform loop with NT2's OpenMP chunking
 *     (modules/arch/shared_memory/include/nt2/core/functions/shared_memory/transform.hpp:36-48,
 *      modules/arch/openmp/include/nt2/sdk/openmp/spawner/transform.hpp:47-72);
 *   - the inner_fold / outer_fold accumulation orders
 *     (modules/core/reduction/include/nt2/core/functions/simd/inner_fold.hpp:49-66,
 *      modules/core/reduction/include/nt2/core/functions/details/outer_fold_step.hpp:33-67);
 *   - NT2's ulpdist
 *     (modules/boost/simd/base/include/boost/simd/ieee/functions/scalar/ulpdist.hpp:64-83).
 *
 * Parity is pinned against NT2's own unit-test values (tests/test_oracle_golden.py).
 * Build: cc -O2 -ffp-contract=off -fopenmp -fPIC -shared (oracle/build_oracle.py).
 * -ffp-contract=off is required: NT2's fma/fnms/horner round twice.
 */
#include <float.h>
#include <stddef.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

static inline float fb(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t bf(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline double db(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static inline uint64_t bd(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

/* ------------------------------------------------------------- ulpdist -- */
/* boost/simd/ieee/functions/scalar/ulpdist.hpp:64-83: |a-b| rescaled by the
 * larger frexp exponent, divided by Eps.  Adjacent floats are 0.5 apart.
 * Infinities: equal infinities are 0, anything else against one is +inf. */
EXPORT double nt2o_ulpdist_f(float a0, float a1)
{
  if (a0 == a1) return 0.0;
  if (isnan(a0) && isnan(a1)) return 0.0;
  if (isnan(a0) || isnan(a1) || isinf(a0) || isinf(a1)) return INFINITY;
  int e1, e2;
  float m1 = frexpf(a0, &e1), m2 = frexpf(a1, &e2);
  int expo = -(e1 > e2 ? e1 : e2);
  float e = (e1 == e2) ? fabsf(m1 - m2) : fabsf(ldexpf(a0, expo) - ldexpf(a1, expo));
  return (double)(e / FLT_EPSILON);
}

EXPORT double nt2o_ulpdist_d(double a0, double a1)
{
  if (a0 == a1) return 0.0;
  if (isnan(a0) && isnan(a1)) return 0.0;
  if (isnan(a0) || isnan(a1) || isinf(a0) || isinf(a1)) return INFINITY;
  int e1, e2;
  double m1 = frexp(a0, &e1), m2 = frexp(a1, &e2);
  int expo = -(e1 > e2 ? e1 : e2);
  double e = (e1 == e2) ? fabs(m1 - m2) : fabs(ldexp(a0, expo) - ldexp(a1, expo));
  return e / DBL_EPSILON;
}

/* Max ulpdist over two arrays, and index of the worst element. */
EXPORT double nt2o_max_ulp_f(const float* a, const float* b, size_t n, size_t* where)
{
  double m = 0.0; size_t w = 0;
  for (size_t i = 0; i < n; ++i) {
    double d = nt2o_ulpdist_f(a[i], b[i]);
    if (d > m) { m = d; w = i; }
  }
  if (where) *where = w;
  return m;
}

EXPORT double nt2o_max_ulp_d(const double* a, const double* b, size_t n, size_t* where)
{
  double m = 0.0; size_t w = 0;
  for (size_t i = 0; i < n; ++i) {
    double d = nt2o_ulpdist_d(a[i], b[i]);
    if (d > m) { m = d; w = i; }
  }
  if (where) *where = w;
  return m;
}

/* ------------------------------------------------------------ constants -- */
/* Float / double bit patterns of the Boost.SIMD / NT2 constants
 * (BOOST_SIMD_CONSTANT_REGISTER lines of each constant's header). */
#define MAXLOG_F      fb(0x42b0c0a5u)   /* exponential/constants/maxlog.hpp:29 */
#define MINLOG_F      fb(0xc2b0c0a5u)   /* exponential/constants/minlog.hpp:29 */
#define INVLOG_2_F    fb(0x3fb8aa3bu)   /* exponential/constants/invlog_2.hpp:29 */
#define LOG_2HI_F     fb(0x3f318000u)   /* exponential/constants/log_2hi.hpp:29 */
#define LOG_2LO_F     fb(0xb95e8083u)   /* exponential/constants/log_2lo.hpp:29 */
#define SQRT_2O_2_F   fb(0x3f3504f3u)   /* boost/simd/constant/constants/sqrt_2o_2.hpp:30 */
#define TWOTHIRD_F    fb(0x3f2aaaabu)   /* boost/simd/constant/constants/twothird.hpp:30 */
#define INVSQRT_2PI_F fb(0x3ecc422au)   /* trigonometric/constants/invsqrt_2pi.hpp:28 */
#define SMALLESTPOSVAL_F fb(0x00800000u)
#define TWOTONMB_F    fb(0x4b000000u)
#define MLOGTWO2NMB_F fb(0xc17f1402u)   /* exponential/constants/mlogtwo2nmb.hpp:29 */

#define MAXLOG_D      db(0x40862e42fefa39efull)
#define MINLOG_D      db(0xc086232bdd7abcd2ull)
#define INVLOG_2_D    db(0x3ff71547652b82feull)
#define LOG_2HI_D     db(0x3fe62e42fee00000ull)
#define LOG_2LO_D     db(0x3dea39ef35793c76ull)
#define SQRT_2O_2_D   db(0x3fe6a09e667f3bcdull)

/* ------------------------------------------------------------- helpers -- */
/* round2even: boost/simd/arithmetic/functions/scalar/round2even.hpp:29-36
 * (the 2^nmb add/subtract trick == round-half-even in the default mode). */
static inline float  r2e_f(float a)  { return rintf(a); }
static inline double r2e_d(double a) { return rint(a); }

/* scale(y,k) = y * 2^k through the exponent bits:
 * exponential/functions/scalar/impl/expo/expo_scale.hpp:26-35 */
static inline float scale_f(float y, float k)
{
  uint32_t ik = (uint32_t)((int32_t)k + 127);
  return y * fb(ik << 23);
}
static inline double scale_d(double y, double k)
{
  uint64_t ik = (uint64_t)((int64_t)k + 1023);
  return y * db(ik << 52);
}

/* fast_frexp: boost/simd/ieee/functions/scalar/fast_frexp.hpp:48-56 */
static inline float frexp_f(float a0, int32_t* e)
{
  uint32_t u = bf(a0);
  *e = (int32_t)((u & 0x7f800000u) >> 23) - 126;
  return fb((u & ~0x7f800000u) | 0x3f000000u);
}
static inline double frexp_d(double a0, int64_t* e)
{
  uint64_t u = bd(a0);
  *e = (int64_t)((u & 0x7ff0000000000000ull) >> 52) - 1022;
  return db((u & ~0x7ff0000000000000ull) | 0x3fe0000000000000ull);
}

/* Static Horner, coefficients in decreasing powers, unfused fma(x,acc,c):
 * polynomials/functions/scalar/impl/horner.hpp:26-45 */
static inline float horner_f(float x, const uint32_t* c, int n)
{
  float acc = fb(c[0]);
  for (int i = 1; i < n; ++i) acc = x * acc + fb(c[i]);
  return acc;
}
static inline double horner_d(double x, const uint64_t* c, int n)
{
  double acc = db(c[0]);
  for (int i = 1; i < n; ++i) acc = x * acc + db(c[i]);
  return acc;
}

/* ------------------------------------------------------------ float exp -- */
/* exponential/functions/scalar/impl/expo/f_expo_reduction.hpp:62-85 (approx,
 * reduce) with the selection order of
 * exponential/functions/simd/common/impl/expo/expo_base.hpp:48-62. */
static const uint32_t EXP_F_P[5] = {0x3ab778cfu, 0x3c098d8bu, 0x3d2aa957u, 0x3e2aa9a5u, 0x3f000000u};

EXPORT float nt2o_exp_f(float a0)
{
  if (isnan(a0)) return a0;
  if (a0 >= MAXLOG_F) return INFINITY;
  if (a0 <= MINLOG_F) return 0.0f;
  float k = r2e_f(INVLOG_2_F * a0);
  float x = a0 - k * LOG_2HI_F;
  x = x - k * LOG_2LO_F;
  float y = horner_f(x, EXP_F_P, 5);
  float c = (y * (x * x) + x) + 1.0f;
  return scale_f(c, k);
}

/* ------------------------------------------------------------ float log -- */
/* exponential/functions/simd/common/impl/logs/f_log.hpp:101-124 + finalize
 * :173-186, kernel exponential/functions/scalar/impl/logs/f_kernel.hpp:43-73 */
static const uint32_t LOG_F_P[8] = {0xbda5dff0u, 0x3e0229f9u, 0xbe04d6b7u, 0x3e116e80u,
                                    0xbe2a6aa0u, 0x3e4cd0a3u, 0xbe800064u, 0x3eaaaaa9u};

EXPORT float nt2o_log_f(float a0)
{
  float z = a0, t = 0.0f;
  if (fabsf(z) < SMALLESTPOSVAL_F) { z = z * TWOTONMB_F; t = MLOGTWO2NMB_F; }
  int32_t e;
  float x = frexp_f(z, &e);
  int lt = x < SQRT_2O_2_F;
  float fe = lt ? ((float)e + -1.0f) : (float)e;
  x = (lt ? x + x : x) - 1.0f;
  float x2 = x * x;
  float y = (horner_f(x, LOG_F_P, 8) * x) * x2;
  y = fe * LOG_2LO_F + y;
  y = -0.5f * x2 + y;
  float r = LOG_2HI_F * fe + ((x + y) + t);
  if (a0 < 0.0f || isnan(a0)) r = NAN;
  if (a0 == INFINITY) r = a0;
  if (a0 == 0.0f) r = -INFINITY;
  return r;
}

/* ----------------------------------------------------------- float erfc -- */
/* euler/functions/simd/common/erfc.hpp:92-121, kernels
 * euler/functions/details/erf_kernel.hpp:48-85 (erfc2 degree 10, erfc3 degree 8) */
static const uint32_t ERFC2_F_P[11] = {0xc0283611u, 0x40d67e3bu, 0xc0cd1a85u, 0x4050b063u,
                                       0xbfaea865u, 0x3e2006f0u, 0x3e1175c7u, 0x3ec4ca6eu,
                                       0x3e243828u, 0xbf918a62u, 0x3f0a0e8bu};
static const uint32_t ERFC3_F_P[9] = {0x41aa8e55u, 0x401b5680u, 0xc010d956u, 0x3f2cff3bu,
                                      0xc016c985u, 0xbffc9284u, 0xbfa11698u, 0xbe036d7eu,
                                      0x3f7ffffeu};

/* erfc of |a0| only (the part shared by erfc(a) and erfc(-a)) */
static inline float erfc_abs_f(float x)
{
  float z = x / (1.0f + x);
  float r1;
  if (x < TWOTHIRD_F) {
    r1 = (1.0f - z) * horner_f(z, ERFC3_F_P, 9);
  } else {
    z = z - 0.4f;
    r1 = nt2o_exp_f(-(x * x)) * horner_f(z, ERFC2_F_P, 11);
  }
  if (x == INFINITY) r1 = 0.0f;
  return r1;
}

EXPORT float nt2o_erfc_f(float a0)
{
  float r1 = erfc_abs_f(fabsf(a0));
  return (a0 < 0.0f) ? 2.0f - r1 : r1;
}

/* normcdf(x) = 0.5*erfc(-sqrt(2)/2*x): statistics/functions/generic/normcdf.hpp:28-34 */
EXPORT float nt2o_normcdf_f(float a0)
{
  return 0.5f * nt2o_erfc_f((-SQRT_2O_2_F) * a0);
}

/* fastnormcdf (Abramowitz-Stegun 26.2.17): statistics/functions/generic/fastnormcdf.hpp:33-53 */
static const uint32_t FNCDF_P[5] = {0x3faa466fu, 0xbfe91eeau, 0x3fe40778u, 0xbeb68f87u, 0x3ea385fau};

EXPORT float nt2o_fastnormcdf_f(float a0)
{
  float l = fabsf(a0);
  float k = 1.0f / (0.2316419f * l + 1.0f);
  float w = horner_f(k, FNCDF_P, 5);
  w = w * ((k * INVSQRT_2PI_F) * nt2o_exp_f((-(l * l)) * 0.5f));
  return (a0 > 0.0f) ? 1.0f - w : w;
}

/* ----------------------------------------------------------- double exp -- */
/* exponential/functions/scalar/impl/expo/d_expo_reduction.hpp:57-82 with the
 * selections of exponential/functions/simd/common/impl/expo/expo_base.hpp:31-45 */
static const uint64_t EXP_D_P[5] = {0x3e66376972bea4d0ull, 0xbebbbd41c5d26bf1ull,
                                    0x3f11566aaf25de2cull, 0xbf66c16c16bebd93ull,
                                    0x3fc555555555553eull};

EXPORT double nt2o_exp_d(double a0)
{
  if (isnan(a0)) return a0;
  if (a0 >= MAXLOG_D) return INFINITY;
  if (a0 <= MINLOG_D) return 0.0;
  double k = r2e_d(INVLOG_2_D * a0);
  double hi = a0 - k * LOG_2HI_D;
  double lo = k * LOG_2LO_D;
  double x = hi - lo;
  double t = x * x;
  double c = x - t * horner_d(t, EXP_D_P, 5);
  c = 1.0 - ((lo - (x * c) / (2.0 - c)) - hi);
  return scale_d(c, k);
}

/* ----------------------------------------------------------- double log -- */
/* exponential/functions/simd/common/impl/logs/d_log.hpp:57-98 + finalize :124-137 */
static const uint64_t LOG_D_T1[3] = {0x3fc39a09d078c69full, 0x3fcc71c51d8e78afull, 0x3fd999999997fa04ull};
static const uint64_t LOG_D_T2[4] = {0x3fc2f112df3e5244ull, 0x3fc7466496cb03deull,
                                     0x3fd2492494229359ull, 0x3fe5555555555593ull};

EXPORT double nt2o_log_d(double a0)
{
  int64_t k;
  double x = frexp_d(a0, &k);
  int lt = SQRT_2O_2_D > x;
  k = k + (lt ? -1 : 0);
  double f = (x + (lt ? x : 0.0)) - 1.0;
  double dk = (double)k;
  double s = f / (2.0 + f);
  double z = s * s;
  double w = z * z;
  double t1 = w * horner_d(w, LOG_D_T1, 3);
  double t2 = z * horner_d(w, LOG_D_T2, 4);
  double R = t2 + t1;
  double hfsq = 0.5 * (f * f);
  double y = dk * LOG_2HI_D - ((hfsq - (s * (hfsq + R) + dk * LOG_2LO_D)) - f);
  if (a0 < 0.0 || isnan(a0)) y = NAN;
  if (a0 == INFINITY) y = a0;
  if (a0 == 0.0) y = -INFINITY;
  return y;
}

/* ------------------------------------------- exp2, exp10, log2, log10 -- */
/* Same skeletons as exp and log with NT2's other reductions and recombinations:
 * exp2/exp10 float: exponential/functions/scalar/impl/expo/f_expo_reduction.hpp:88-143,
 * double: d_expo_reduction.hpp:85-160, selections simd/common/impl/expo/expo_base.hpp:26-65;
 * log2/log10 float: simd/common/impl/logs/f_log.hpp:126-170, double:
 * simd/common/impl/logs/d_log.hpp:99-121.  Constants: the headers of exponential/constants. */
#define MAXLOG2_F     fb(0x42fe0000u)
#define MINLOG2_F     fb(0xc2fe0000u)
#define MAXLOG10_F    fb(0x4218ec59u)
#define MINLOG10_F    fb(0xc2179999u)
#define INVLOG10_2_F  fb(0x40549a78u)
#define LOG10_2HI_F   fb(0x3e9a0000u)
#define LOG10_2LO_F   fb(0x39826a14u)
#define LOG_2_F       fb(0x3f317218u)
#define LOG2_EM1_F    fb(0x3ee2a8edu)
#define LOG10_ELO_F   fb(0x3a37b152u)
#define LOG10_EHI_F   fb(0x3ede0000u)
#define MLOG2TWO2NMB_F  fb(0xc1b80000u)
#define MLOG10TWO2NMB_F fb(0xc0dd8edeu)
#define MAXLOG2_D     db(0x408ff80000000000ull)
#define MINLOG2_D     db(0xc08ff00000000000ull)
#define MAXLOG10_D    db(0x40734413509f79feull)
#define MINLOG10_D    db(0xc0734413509f79feull)
#define INVLOG10_2_D  db(0x400a934f0979a372ull)
#define LOG10_2HI_D   db(0x3fd3440000000000ull)
#define LOG10_2LO_D   db(0x3ed3509f79fef312ull)
#define LOG_2_D       db(0x3fe62e42fefa39efull)
#define INVLOG_10_D   db(0x3fdbcb7b1526e50dull)
#define LOG_2OLOG_10_D db(0x3fd34413509f79ffull)

static const uint32_t EXP2_F_P[5] = {0x3922c8c4u, 0x3ab01218u, 0x3c1d9422u, 0x3d6356ebu, 0x3e75fdf1u};
static const uint32_t EXP10_F_P[6] = {0x3e54dff1u, 0x3f0aacefu, 0x3f95eb4cu, 0x400237dau, 0x4029a926u, 0x40135d8eu};
static const uint64_t EXP10_D_P[4] = {0x3fa4fd75f3062dd4ull, 0x40277d9474c55934ull, 0x40796b7a050349e4ull,
                                      0x40a2b4798e134a01ull};
static const uint64_t EXP10_D_Q[4] = {0x3ff0000000000000ull, 0x405545fdce51ca08ull, 0x4093e05eefd67782ull,
                                      0x40a03f37650df6e2ull};

/* the guards of expo_base: NaN -> NaN, >= maxlog -> Inf, <= minlog -> 0, else scale(c, k) */
static inline float expo_select_f(float a0, float c, float k, float minl, float maxl)
{
  if (isnan(a0)) return a0;
  if (a0 >= maxl) return INFINITY;
  if (a0 <= minl) return 0.0f;
  return scale_f(c, k);
}
static inline double expo_select_d(double a0, double c, double k, double minl, double maxl)
{
  if (isnan(a0)) return a0;
  if (a0 >= maxl) return INFINITY;
  if (a0 <= minl) return 0.0;
  return scale_d(c, k);
}

EXPORT float nt2o_exp2_f(float a0)
{
  float k = r2e_f(a0);
  float x = a0 - k;
  float y = horner_f(x, EXP2_F_P, 5);
  float c = (y * (x * x) + x * LOG_2_F) + 1.0f;           /* inc(fma(y, sqr(x), x*Log_2)) */
  return expo_select_f(a0, c, k, MINLOG2_F, MAXLOG2_F);
}

EXPORT float nt2o_exp10_f(float a0)
{
  float k = r2e_f(INVLOG10_2_F * a0);
  float x = a0 - k * LOG10_2HI_F;                          /* fnms(k, Log10_2hi, a0) */
  x = x - k * LOG10_2LO_F;
  float c = horner_f(x, EXP10_F_P, 6) * x + 1.0f;          /* inc(horner(x)*x) */
  return expo_select_f(a0, c, k, MINLOG10_F, MAXLOG10_F);
}

EXPORT double nt2o_exp2_d(double a0)
{
  double k = r2e_d(a0);
  double x = (a0 - k) * LOG_2_D;
  double t = x * x;
  double c = x - t * horner_d(t, EXP_D_P, 5);             /* approx: fnms(t, horner(t), x) */
  c = 1.0 - ((-(x * c) / (2.0 - c)) - x);                  /* finalize: oneminus(...) */
  return expo_select_d(a0, c, k, MINLOG2_D, MAXLOG2_D);
}

EXPORT double nt2o_exp10_d(double a0)
{
  double k = r2e_d(INVLOG10_2_D * a0);
  double x = a0 - k * LOG10_2HI_D;
  x = x - k * LOG10_2LO_D;
  double xx = x * x;
  double px = x * horner_d(xx, EXP10_D_P, 4);
  double x2 = px / (horner_d(xx, EXP10_D_Q, 4) - px);
  double c = (x2 + x2) + 1.0;                              /* oneplus(x2+x2) */
  return expo_select_d(a0, c, k, MINLOG10_D, MAXLOG10_D);
}

/* the float log kernel (f_kernel.hpp:43-73) after the denormal rescale of f_log.hpp */
static inline void log_kernel_f(float a0, float mtwo2nmb, float* fe, float* x, float* x2, float* y, float* t)
{
  float z = a0;
  *t = 0.0f;
  if (fabsf(z) < SMALLESTPOSVAL_F) { z = z * TWOTONMB_F; *t = mtwo2nmb; }
  int32_t e;
  float m = frexp_f(z, &e);
  int lt = m < SQRT_2O_2_F;
  *fe = lt ? ((float)e + -1.0f) : (float)e;
  *x = (lt ? m + m : m) - 1.0f;
  *x2 = *x * *x;
  *y = (horner_f(*x, LOG_F_P, 8) * *x) * *x2;
}

static inline float log_finalize_f(float a0, float r)
{
  if (a0 < 0.0f || isnan(a0)) r = NAN;
  if (a0 == INFINITY) r = a0;
  if (a0 == 0.0f) r = -INFINITY;
  return r;
}

EXPORT float nt2o_log2_f(float a0)
{
  float fe, x, x2, y, t;
  log_kernel_f(a0, MLOG2TWO2NMB_F, &fe, &x, &x2, &y, &t);
  y = -0.5f * x2 + y;                                      /* fma(Mhalf, x2, y) */
  float z = x * LOG2_EM1_F + y * LOG2_EM1_F;               /* fma(x, Log2_em1, y*Log2_em1) */
  return log_finalize_f(a0, (((z + y) + x) + fe) + t);
}

EXPORT float nt2o_log10_f(float a0)
{
  float fe, x, x2, y, t;
  log_kernel_f(a0, MLOG10TWO2NMB_F, &fe, &x, &x2, &y, &t);
  y = -0.5f * x2 + y;                                      /* amul(y, Mhalf, x2) */
  float z = (x + y) * LOG10_ELO_F;
  z = y * LOG10_EHI_F + z;                                 /* amul(z, y, Log10_ehi) */
  z = x * LOG10_EHI_F + z;
  z = fe * LOG10_2HI_F + z;
  return log_finalize_f(a0, fe * LOG10_2LO_F + (z + t));   /* amul(z+t, fe, Log10_2lo) */
}

/* the double log kernel of d_log.hpp:57-87 */
static inline void log_kernel_d(double a0, double* dk, double* hfsq, double* s, double* R, double* f)
{
  int64_t k;
  double x = frexp_d(a0, &k);
  int lt = SQRT_2O_2_D > x;
  k = k + (lt ? -1 : 0);
  *f = (x + (lt ? x : 0.0)) - 1.0;
  *dk = (double)k;
  *s = *f / (2.0 + *f);
  double z = *s * *s;
  double w = z * z;
  double t1 = w * horner_d(w, LOG_D_T1, 3);
  double t2 = z * horner_d(w, LOG_D_T2, 4);
  *R = t2 + t1;
  *hfsq = 0.5 * (*f * *f);
}

static inline double log_finalize_d(double a0, double y)
{
  if (a0 < 0.0 || isnan(a0)) y = NAN;
  if (a0 == INFINITY) y = a0;
  if (a0 == 0.0) y = -INFINITY;
  return y;
}

EXPORT double nt2o_log2_d(double a0)
{
  double dk, hfsq, s, R, f;
  log_kernel_d(a0, &dk, &hfsq, &s, &R, &f);
  double y = (-((hfsq - s * (hfsq + R)) - f)) * INVLOG_2_D + dk;
  return log_finalize_d(a0, y);
}

EXPORT double nt2o_log10_d(double a0)
{
  double dk, hfsq, s, R, f;
  log_kernel_d(a0, &dk, &hfsq, &s, &R, &f);
  double y = (-((hfsq - s * (hfsq + R)) - f)) * INVLOG_10_D + dk * LOG_2OLOG_10_D;
  return log_finalize_d(a0, y);
}

/* ------------------------------------------------------- expm1, log1p -- */
/* expm1: exponential/functions/details/expm1_kernel.hpp:24-80 with the
 * selections of simd/common/expm1.hpp:35-41 (below Logeps: -1, above Maxlog:
 * Inf); fast_ldexp multiplies by 2^ik built in the exponent bits
 * (boost/simd/ieee/functions/simd/common/fast_ldexp.hpp).
 * log1p: simd/common/log1p.hpp:29-38, u = 1+a0, log(u) corrected by (a0-(u-1))/u. */
#define LOGEPS_F fb(0xc17f1402u)
#define LOGEPS_D db(0xc04205966f2b4f19ull)
static const uint32_t EXPM1_F_P[3] = {0x3acf6db4u, 0xbd08887fu, 0x3f800000u};
static const uint64_t EXPM1_D_P[6] = {0xBE8AFDB76E09C32Dull, 0x3ED0CFCA86E65239ull, 0xBF14CE199EAADBB7ull,
                                      0x3F5A01A019FE5585ull, 0xBFA11111111110F4ull, 0x3ff0000000000000ull};

EXPORT float nt2o_expm1_f(float a0)
{
  if (a0 < LOGEPS_F) return -1.0f;
  if (a0 > MAXLOG_F) return INFINITY;
  float k = r2e_f(INVLOG_2_F * a0);
  float x = a0 - k * LOG_2HI_F;
  x = x - k * LOG_2LO_F;
  float hx = x * 0.5f;
  float hxs = x * hx;
  float r1 = horner_f(hxs, EXPM1_F_P, 3);
  float t = 3.0f - r1 * hx;                                 /* fnms(r1, hx, Three) */
  float e = hxs * ((r1 - t) / (6.0f - x * t));
  e = x * e - hxs;                                          /* fms(x, e, hxs) */
  uint32_t ik = (uint32_t)(int32_t)k;                       /* k is integral (NaN only when a0 is) */
  float two2mk = fb((127u - ik) << 23);
  float y = (1.0f - two2mk) - (e - x);
  return y * fb((ik + 127u) << 23);
}

EXPORT double nt2o_expm1_d(double a0)
{
  if (a0 < LOGEPS_D) return -1.0;
  if (a0 > MAXLOG_D) return INFINITY;
  double k = r2e_d(INVLOG_2_D * a0);
  double hi = a0 - k * LOG_2HI_D;
  double lo = k * LOG_2LO_D;
  double x = hi - lo;
  double hxs = (x * x) * 0.5;
  double r1 = horner_d(hxs, EXPM1_D_P, 6);
  double t = 3.0 - (r1 * 0.5) * x;
  double e = hxs * ((r1 - t) / (6.0 - x * t));
  double c = (hi - x) - lo;
  e = (x * (e - c) - c) - hxs;
  uint64_t ik = (uint64_t)(int64_t)k;
  double two2mk = db((1023ull - ik) << 52);
  double ct1 = (1.0 - two2mk) - (e - x);
  double ct2 = (x - (e + two2mk)) + 1.0;
  double y = (k < 20.0) ? ct1 : ct2;
  return y * db((ik + 1023ull) << 52);
}

EXPORT float nt2o_log1p_f(float a0)
{
  float u = 1.0f + a0;
  float r = nt2o_log_f(u);
  if (u != 0.0f) r = r + (a0 - (u - 1.0f)) / u;
  return (u == INFINITY) ? u : r;
}

EXPORT double nt2o_log1p_d(double a0)
{
  double u = 1.0 + a0;
  double r = nt2o_log_d(u);
  if (u != 0.0) r = r + (a0 - (u - 1.0)) / u;
  return (u == INFINITY) ? u : r;
}

/* ---------------------------------------------------------- double erfc -- */
/* euler/functions/simd/common/erfc.hpp:46-89, kernels
 * euler/functions/details/erf_kernel.hpp:101-163 (rational 5/5, 7/7, 7/7) */
static const uint64_t ERF1_D_P[5] = {0x3f110512d5b20332ull, 0x3f53b7664358865aull, 0x3fa4a59a4f02579cull,
                                     0x3fc16500f106c0a5ull, 0x3ff20dd750429b61ull};
static const uint64_t ERF1_D_Q[5] = {0x3f37ea4332348252ull, 0x3f8166f75999dbd1ull, 0x3fb64536ca92ea2full,
                                     0x3fdd0a84eb1ca867ull, 0x3ff0000000000000ull};
static const uint64_t ERFC2_D_P[7] = {0x0ull, 0x3f7cf4cfe0aacbb4ull, 0x3fb2488a6b5cb5e5ull, 0x3fd53dd7a67c7e9full,
                                      0x3fec1986509e687bull, 0x3ff54dfe9b258a60ull, 0x3feffffffbbb552bull};
static const uint64_t ERFC2_D_Q[7] = {0x3f89a996639b0d00ull, 0x3fc033c113a7deeeull, 0x3fe307622fcff772ull,
                                      0x3ff9e677c2777c3cull, 0x40053b1052dca8bdull, 0x4003adeae79b9708ull,
                                      0x3ff0000000000000ull};
static const uint64_t ERFC3_D_P[7] = {0x0ull, 0x3f971d0907ea7a92ull, 0x3fc42210f88b9d43ull, 0x3fe29be1cff90d94ull,
                                      0x3ff44744306832aeull, 0x3ff9fa202deb88e5ull, 0x3fefff5a9e697ae2ull};
static const uint64_t ERFC3_D_Q[7] = {0x3fa47bd61bbb3843ull, 0x3fd1d7ab774bb837ull, 0x3ff0cfd4cb6cde9full,
                                      0x400315ffdfd5ce91ull, 0x400afd487397568full, 0x400602f24bf3fdb6ull,
                                      0x3ff0000000000000ull};

static inline double erfc_abs_d(double x)
{
  double xx = x * x;
  double r1;
  if (x < 0.65) {
    r1 = 1.0 - x * (horner_d(xx, ERF1_D_P, 5) / horner_d(xx, ERF1_D_Q, 5));
  } else {
    double ex = nt2o_exp_d(-xx);
    if (x < 2.2) r1 = ex * (horner_d(x, ERFC2_D_P, 7) / horner_d(x, ERFC2_D_Q, 7));
    else         r1 = ex * (horner_d(x, ERFC3_D_P, 7) / horner_d(x, ERFC3_D_Q, 7));
  }
  if (x == INFINITY) r1 = 0.0;
  return r1;
}

EXPORT double nt2o_erfc_d(double a0)
{
  double r1 = erfc_abs_d(fabs(a0));
  return (a0 < 0.0) ? 2.0 - r1 : r1;
}

EXPORT double nt2o_normcdf_d(double a0)
{
  return 0.5 * nt2o_erfc_d((-SQRT_2O_2_D) * a0);
}

/* ------------------------------------------------- scalar-tail variants -- */
/* NT2's transform runs the SIMD body on N-lane packs and the scalar functor
 * on the n%N tail (core/functions/simd/transform.hpp:46-56).  The scalar
 * erfc forms differ from the SIMD ones; they are restated here so tests can
 * show where the two agree.  euler/functions/scalar/erfc.hpp:38-96. */
EXPORT float nt2o_erfc_f_scalar(float a0)
{
  float x = fabsf(a0);
  float r1 = 0.0f;
  float z = x / (1.0f + x);
  if (x < TWOTHIRD_F) r1 = (1.0f - z) * horner_f(z, ERFC3_F_P, 9);
  else if (x == INFINITY) r1 = 0.0f;
  else { z -= 0.4f; r1 = nt2o_exp_f(-(x * x)) * horner_f(z, ERFC2_F_P, 11); }
  return (a0 < 0.0f) ? 2.0f - r1 : r1;
}

EXPORT double nt2o_erfc_d_scalar(double a0)
{
  if (isnan(a0)) return a0;
  double x = fabs(a0), xx = x * x, z = 0.0;
  if (x <= 0.0000000001) z = 1.0 - x * 2.0 / sqrt(3.14159265358979323846);
  else if (x < 0.65) z = 1.0 - x * (horner_d(xx, ERF1_D_P, 5) / horner_d(xx, ERF1_D_Q, 5));
  else if (x < 2.2) z = nt2o_exp_d(-xx) * (horner_d(x, ERFC2_D_P, 7) / horner_d(x, ERFC2_D_Q, 7));
  else if (x < 6.0) z = nt2o_exp_d(-xx) * (horner_d(x, ERFC3_D_P, 7) / horner_d(x, ERFC3_D_Q, 7));
  return (a0 < 0.0) ? 2.0 - z : z;
}

/* ----------------------------------------------------- sinh, cosh, tanh -- */
/* Paths relative to modules/core/hyperbolic/include/nt2/hyperbolic/functions/:
 * sinh simd/common/sinh.hpp:20-45 (kernel details/sinh_kernel.hpp), cosh
 * generic/cosh.hpp:20-42, tanh simd/common/tanh.hpp:20-48 (kernel
 * details/tanh_kernel.hpp).  The SIMD forms select per lane: no pack dependence.
 * average(a, b) = fma(a, 0.5, b*0.5) (boost/simd/arithmetic/functions/generic/average.hpp). */
static const uint32_t SINH_F_P[4] = {0x39559e2fu, 0x3c087bbeu, 0x3e2aaaccu, 0x3f800000u};
static const uint64_t SINH_D_P[4] = {0xbfe9435fe8bb3cd6ull, 0xc064773a398ff4feull, 0xc0c694b8c71d6182ull,
                                     0xc115782bdbf6ab05ull};
static const uint64_t SINH_D_Q[4] = {0x3ff0000000000000ull, 0xc0715b6096e96484ull, 0x40e1a7ba7ed72245ull,
                                     0xc1401a20e4f90044ull};
static const uint32_t TANH_F_P[5] = {0xbbbaf0eau, 0x3ca9134eu, 0xbd5c1e2du, 0x3e088393u, 0xbeaaaa99u};
static const uint64_t TANH_D_P[3] = {0xbfeedc5baafd6f4bull, 0xc058d26a0e26682dull, 0xc0993ac030580563ull};
static const uint64_t TANH_D_Q[4] = {0x3ff0000000000000ull, 0x405c33f28a581b86ull, 0x40a176fa0e5535faull,
                                     0x40b2ec102442040cull};

EXPORT float nt2o_sinh_f(float a0)
{
  const float x = fabsf(a0);
  const uint32_t bts = bf(a0) & 0x80000000u;
  float r;
  if (x < 1.0f) {
    r = horner_f(x * x, SINH_F_P, 4) * x;
  } else {
    const int test1 = x > MAXLOG_F - LOG_2_F;
    const float tmp = nt2o_exp_f(x * (test1 ? 0.5f : 1.0f));
    const float tmp1 = 0.5f * tmp;
    r = test1 ? tmp1 * tmp : tmp1 - 0.5f * (1.0f / tmp);
  }
  return fb(bf(r) ^ bts);
}
EXPORT double nt2o_sinh_d(double a0)
{
  const double x = fabs(a0);
  const uint64_t bts = bd(a0) & 0x8000000000000000ull;
  double r;
  if (x < 1.0) {
    const double x2 = x * x;
    r = x * (x2 * horner_d(x2, SINH_D_P, 4) / horner_d(x2, SINH_D_Q, 4)) + x;
  } else {
    const int test1 = x > MAXLOG_D - LOG_2_D;
    const double tmp = nt2o_exp_d(x * (test1 ? 0.5 : 1.0));
    const double tmp1 = 0.5 * tmp;
    r = test1 ? tmp1 * tmp : tmp1 - 0.5 * (1.0 / tmp);
  }
  return db(bd(r) ^ bts);
}
EXPORT float nt2o_cosh_f(float a0)
{
  const float x = fabsf(a0);
  const int test1 = x > MAXLOG_F - LOG_2_F;
  const float tmp = nt2o_exp_f(x * (test1 ? 0.5f : 1.0f));
  return test1 ? (0.5f * tmp) * tmp : tmp * 0.5f + (1.0f / tmp) * 0.5f;
}
EXPORT double nt2o_cosh_d(double a0)
{
  const double x = fabs(a0);
  const int test1 = x > MAXLOG_D - LOG_2_D;
  const double tmp = nt2o_exp_d(x * (test1 ? 0.5 : 1.0));
  return test1 ? (0.5 * tmp) * tmp : tmp * 0.5 + (1.0 / tmp) * 0.5;
}
EXPORT float nt2o_tanh_f(float a0)
{
  const float x = fabsf(a0);
  const uint32_t bts = bf(a0) & 0x80000000u;
  float r;
  if (x < 0.625f) {
    const float x2 = x * x;
    r = (horner_f(x2, TANH_F_P, 5) * x2) * x + x;
  } else {
    r = -2.0f * (1.0f / (1.0f + nt2o_exp_f(x + x))) + 1.0f;
  }
  return fb(bf(r) ^ bts);
}
EXPORT double nt2o_tanh_d(double a0)
{
  const double x = fabs(a0);
  const uint64_t bts = bd(a0) & 0x8000000000000000ull;
  double r;
  if (x < 0.625) {
    const double x2 = x * x;
    r = (x2 * horner_d(x2, TANH_D_P, 3) / horner_d(x2, TANH_D_Q, 4)) * x + x;
  } else {
    r = -2.0 * (1.0 / (1.0 + nt2o_exp_d(x + x))) + 1.0;
  }
  return db(bd(r) ^ bts);
}

/* coth and sinhc, NT2's SIMD forms (hyperbolic/functions/simd/common/coth.hpp:32-48,
 * sinhc.hpp:32-56; kernels details/tanh_kernel.hpp:40-58, sinhc_kernel.hpp:25-57):
 * coth: |x| < 5/8 -> rec of the tanh kernel (float) or q/(x*(p*x2 + q)) (double), else
 * 2*rec(exp(2|x|) - 1) + 1; sign of x.  sinhc: |x| < 1 -> the sinh kernel's polynomial
 * (float) or 1 + x2*p/q (double), else exp-based as sinh, divided by |x|. */
EXPORT float nt2o_coth_f(float a0)
{
  const float x = fabsf(a0), x2 = x * x;
  const float z = 1.0f / ((horner_f(x2, TANH_F_P, 5) * x2) * x + x);
  const float r = 2.0f * (1.0f / (nt2o_exp_f(x + x) - 1.0f)) + 1.0f;
  return fb(bf(x < 0.625f ? z : r) ^ (bf(a0) & 0x80000000u));
}
EXPORT double nt2o_coth_d(double a0)
{
  const double x = fabs(a0), x2 = x * x;
  const double q = horner_d(x2, TANH_D_Q, 4);
  const double z = q / (x * (horner_d(x2, TANH_D_P, 3) * x2 + q));
  const double r = 2.0 * (1.0 / (nt2o_exp_d(x + x) - 1.0)) + 1.0;
  return db(bd(x < 0.625 ? z : r) ^ (bd(a0) & 0x8000000000000000ull));
}
EXPORT float nt2o_sinhc_f(float a0)
{
  const float x = fabsf(a0);
  const float z = horner_f(x * x, SINH_F_P, 4);
  const int test1 = x > MAXLOG_F - LOG_2_F;
  const float tmp = nt2o_exp_f(x * (test1 ? 0.5f : 1.0f));
  const float tmp1 = (0.5f * tmp) / x;
  float r = test1 ? tmp1 * tmp : (tmp * 0.5f + (-(1.0f / tmp)) * 0.5f) / x;
  r = x == INFINITY ? x : r;
  return x < 1.0f ? z : r;
}
EXPORT double nt2o_sinhc_d(double a0)
{
  const double x = fabs(a0), x2 = x * x;
  const double z = 1.0 + x2 * horner_d(x2, SINH_D_P, 4) / horner_d(x2, SINH_D_Q, 4);
  const int test1 = x > MAXLOG_D - LOG_2_D;
  const double tmp = nt2o_exp_d(x * (test1 ? 0.5 : 1.0));
  const double tmp1 = (0.5 * tmp) / x;
  double r = test1 ? tmp1 * tmp : (tmp * 0.5 + (-(1.0 / tmp)) * 0.5) / x;
  r = x == INFINITY ? x : r;
  return x < 1.0 ? z : r;
}

/* ------------------------------------------------ inverse hyperbolic -- */
/* atanh and acosh, NT2's SIMD forms (modules/core/hyperbolic/include/nt2/hyperbolic/functions/
 * simd/common/atanh.hpp:38-47, acosh.hpp:36-43); seladd(c, a, b) = a + (c ? b : 0).
 * sech = rec(cosh), csch = rec(sinh), acoth = atanh(rec), asech = acosh(rec) (generic headers). */
EXPORT float nt2o_atanh_f(float a0)
{
  const float ax = fabsf(a0), t = ax + ax, z1 = 1.0f - ax;
  const int test = ax < 0.5f;
  const float tmp = (test ? ax : t) / z1;
  const float r = 0.5f * nt2o_log1p_f(test ? t * tmp + t : tmp);
  return fb(bf(r) ^ (bf(a0) & 0x80000000u));
}
EXPORT double nt2o_atanh_d(double a0)
{
  const double ax = fabs(a0), t = ax + ax, z1 = 1.0 - ax;
  const int test = ax < 0.5;
  const double tmp = (test ? ax : t) / z1;
  const double r = 0.5 * nt2o_log1p_d(test ? t * tmp + t : tmp);
  return db(bd(r) ^ (bd(a0) & 0x8000000000000000ull));
}
EXPORT float nt2o_acosh_f(float a0)
{
  const float t = a0 - 1.0f;
  const int test = t > fb(0x4a800000u);                 /* Oneotwoeps */
  const float z = test ? a0 : t + sqrtf((t + t) + t * t);
  return nt2o_log1p_f(z) + (test ? LOG_2_F : 0.0f);
}
EXPORT double nt2o_acosh_d(double a0)
{
  const double t = a0 - 1.0;
  const int test = t > db(0x4320000000000000ull);
  const double z = test ? a0 : t + sqrt((t + t) + t * t);
  return nt2o_log1p_d(z) + (test ? LOG_2_D : 0.0);
}

/* ------------------------------------------------------------------ pow -- */
/* pow(a0, a1) for floating a1, NT2's SIMD form: exponential/functions/simd/common/pow.hpp:20-29
 * over pow_abs (simd/common/pow_abs.hpp:23-79, the cephes algorithm with 2^(-i/16) tables in
 * details/pow_kernel.hpp), frexp and ldexp of Boost.SIMD
 * (boost/simd/ieee/functions/simd/common/{frexp,ldexp}.hpp).  POW_A* are 2^(-i/16) rounded
 * to the type, POW_B* the rounding residuals of the even entries (2^(-2k/16) - A[2k]). */
static const uint32_t POW_AF[17] = {0x3f800000u, 0x3f75257du, 0x3f6ac0c7u, 0x3f60ccdfu, 0x3f5744fdu, 0x3f4e248cu,
                                    0x3f45672au, 0x3f3d08a4u, 0x3f3504f3u, 0x3f2d583fu, 0x3f25fed7u, 0x3f1ef532u,
                                    0x3f1837f0u, 0x3f11c3d3u, 0x3f0b95c2u, 0x3f05aac3u, 0x3f000000u};
static const uint32_t POW_BF[9] = {0x00000000u, 0xb1c116deu, 0xb254a58au, 0x318aa837u, 0x324fe77au, 0xb2ac9d5eu,
                                   0x32a31b71u, 0xb1e0aba1u, 0x00000000u};
static const uint64_t POW_AD[17] = {0x3ff0000000000000ull, 0x3feea4afa2a490daull, 0x3fed5818dcfba487ull,
                                    0x3fec199bdd85529cull, 0x3feae89f995ad3adull, 0x3fe9c49182a3f090ull,
                                    0x3fe8ace5422aa0dbull, 0x3fe7a11473eb0187ull, 0x3fe6a09e667f3bcdull,
                                    0x3fe5ab07dd485429ull, 0x3fe4bfdad5362a27ull, 0x3fe3dea64c123422ull,
                                    0x3fe306fe0a31b715ull, 0x3fe2387a6e756238ull, 0x3fe172b83c7d517bull,
                                    0x3fe0b5586cf9890full, 0x3fe0000000000000ull};
static const uint64_t POW_BD[9] = {0x0000000000000000ull, 0x3c72ed02d75b3707ull, 0x3c87a1cd345dcc81ull,
                                   0x3c86e9f156864b27ull, 0xbc8bdd3413b26456ull, 0x3c6d4397afec42e2ull,
                                   0x3c76f46ad23182e4ull, 0xbc719041b9d78a76ull, 0x0000000000000000ull};
static const uint32_t POW1_F[4] = {0xbe2a61b2u, 0x3e4d2fa3u, 0xbe800015u, 0x3eaaaaa3u};
static const uint32_t POW2_F[4] = {0x3c1a49bcu, 0x3d634d38u, 0x3e75fde1u, 0x3f317218u};
static const uint64_t POW1_DP[4] = {0x3fdfdb997f5b5cf0ull, 0x400dddefea9edf15ull, 0x401eccbd7f78eb6full,
                                    0x4012aa83b65c9b74ull};
static const uint64_t POW1_DQ[5] = {0x3ff0000000000000ull, 0x4022aab49b20914eull, 0x403bffff41c1c9f5ull,
                                    0x4040ccbc1b176402ull, 0x402bffc5918ae92eull};
static const uint64_t POW2_D[7] = {0x3eef6307d7f2937full, 0x3f242fbe60fc9259ull, 0x3f55d87ec84aef1dull,
                                   0x3f83b2ab6ef133b7ull, 0x3fac6b08d7041a92ull, 0x3fcebfbdff82c56dull,
                                   0x3fe62e42fefa39efull};
#define LOG2_EM1_D 0x3fdc551d94ae0bf8ull
#define POWLARGE_F 0x44ffe000u
#define POWLOW_F   0xc5160000u
#define POWLARGE_D 0x40cfff8000000000ull
#define POWLOW_D   0xc0d0c7c000000000ull

static inline int clamp16(int64_t i) { return i < 0 ? 0 : (i > 16 ? 16 : (int)i); }
static inline int32_t sat_i32(double w) { return (w != w) ? 0 : (w >= 2147483647.0 ? INT32_MAX : (w <= -2147483648.0 ? INT32_MIN : (int32_t)w)); }
static inline int64_t sat_i64(double w)
{
  return (w != w) ? 0 : (w >= 9.2e18 ? INT64_MAX : (w <= -9.2e18 ? INT64_MIN : (int64_t)w));
}

static float pow_frexp_f(float a0, int32_t* e)
{
  const int den = fabsf(a0) < fb(0x00800000u) && a0 != 0.0f;
  const float aa0 = den ? 8388608.0f * a0 : a0;
  const int32_t t = den ? 23 : 0;
  const uint32_t b = bf(aa0);
  int32_t r1 = (int32_t)((b & 0x7f800000u) >> 23) - 126;
  float r0 = fb((b & ~0x7f800000u) | 0x3f000000u);
  const int test0 = aa0 != 0.0f, test1 = r1 > 128;
  r1 = (!test1 && test0) ? r1 : 0;
  r1 -= t;
  r0 = test0 ? r0 + (test1 ? aa0 : 0.0f) : 0.0f;
  *e = r1;
  return r0;
}
static float pow_ldexp_f(float a0, int32_t e)
{
  float f = 1.0f;
  const int den = e < -126;
  e = den ? e + 126 : e;
  f = den ? fb(0x00800000u) : 1.0f;
  const int test = e == 128;
  f = f + (test ? 1.0f : 0.0f);
  e = e - (test ? 1 : 0);
  const uint32_t bits = ((uint32_t)(e + 127)) << 23;
  return (a0 * fb(bits)) * f;
}
static double pow_frexp_d(double a0, int64_t* e)
{
  const int den = fabs(a0) < db(0x0010000000000000ull) && a0 != 0.0;
  const double aa0 = den ? 4503599627370496.0 * a0 : a0;
  const int64_t t = den ? 52 : 0;
  const uint64_t b = bd(aa0);
  int64_t r1 = (int64_t)((b & 0x7ff0000000000000ull) >> 52) - 1022;
  double r0 = db((b & ~0x7ff0000000000000ull) | 0x3fe0000000000000ull);
  const int test0 = aa0 != 0.0, test1 = r1 > 1024;
  r1 = (!test1 && test0) ? r1 : 0;
  r1 -= t;
  r0 = test0 ? r0 + (test1 ? aa0 : 0.0) : 0.0;
  *e = r1;
  return r0;
}
static double pow_ldexp_d(double a0, int64_t e)
{
  double f = 1.0;
  const int den = e < -1022;
  e = den ? e + 1022 : e;
  f = den ? db(0x0010000000000000ull) : 1.0;
  const int test = e == 1024;
  f = f + (test ? 1.0 : 0.0);
  e = e - (test ? 1 : 0);
  const uint64_t bits = ((uint64_t)(e + 1023)) << 52;
  return (a0 * db(bits)) * f;
}
static inline float reduc_f(float x) { return 0.0625f * floorf(16.0f * x); }
static inline double reduc_d(double x) { return 0.0625 * floor(16.0 * x); }

/* pow_kernel<float>::select: x <- (x - A[i] - B[i/2]) / A[i] */
static int pow_select_f(float* xp)
{
  float x = *xp;
  int i = 1;
  i = (x <= fb(POW_AF[9])) ? 9 : i;
  i = i + ((x <= fb(POW_AF[clamp16(i + 4)])) ? 4 : 0);
  i = i + ((x <= fb(POW_AF[clamp16(i + 2)])) ? 2 : 0);
  i = (x >= fb(POW_AF[1])) ? -1 : i;
  i = i + 1;
  const float tmp = fb(POW_AF[i]);
  x -= tmp;
  x -= fb(POW_BF[i >> 1]);
  x /= tmp;
  *xp = x;
  return i;
}
static int pow_select_d(double* xp)
{
  double x = *xp;
  int i = 1;
  i = (x <= db(POW_AD[9])) ? 9 : i;
  i = i + ((x <= db(POW_AD[clamp16(i + 4)])) ? 4 : 0);
  i = i + ((x <= db(POW_AD[clamp16(i + 2)])) ? 2 : 0);
  i = (x >= db(POW_AD[1])) ? -1 : i;
  i = i + 1;
  const double tmp = db(POW_AD[i]);
  x -= tmp;
  x -= db(POW_BD[i >> 1]);
  x /= tmp;
  *xp = x;
  return i;
}

static float pow_abs_f(float a0, float a1)
{
  int32_t e;
  const float ax = fabsf(a0);
  float x = pow_frexp_f(ax, &e);
  int32_t i = pow_select_f(&x);
  float z = x * x;
  float w = (z * x) * horner_f(x, POW1_F, 4);
  w = -0.5f * z + w;
  w = LOG2_EM1_F * w + w;
  z = LOG2_EM1_F * x + w;
  z += x;
  w = (float)(-i) * 0.0625f + (float)e;
  const float ya = reduc_f(a1);
  const float yb = a1 - ya;
  float W = z * a1 + w * yb;
  float Wa = reduc_f(W);
  float Wb = W - Wa;
  W = w * ya + Wa;
  Wa = reduc_f(W);
  const float u = W - Wa;
  W = Wb + u;
  Wb = reduc_f(W);
  w = 16.0f * (Wa + Wb);
  const int inf_ret = w > fb(POWLARGE_F), zer_ret = w < fb(POWLOW_F);
  e = sat_i32(w);
  Wb = W - Wb;
  const int test = Wb > 0.0f;
  e = test ? e + 1 : e;
  Wb = Wb - (test ? 0.0625f : 0.0f);
  z = horner_f(Wb, POW2_F, 4) * Wb;
  i = (e > 0) ? e / 16 + 1 : e / 16;
  e = i * 16 - e;
  w = fb(POW_AF[clamp16(e)]);
  z = w * z + w;
  z = pow_ldexp_f(z, i);
  const int gtax1 = ax > 1.0f;
  z = (a1 == INFINITY) ? (gtax1 ? INFINITY : 0.0f) : z;
  z = (a1 == -INFINITY) ? (gtax1 ? 0.0f : INFINITY) : z;
  z = (ax == INFINITY) ? (a1 > 0.0f ? INFINITY : (a1 < 0.0f ? 0.0f : 1.0f)) : z;
  z = zer_ret ? 0.0f : z;
  z = inf_ret ? INFINITY : z;
  z = (ax == 1.0f) ? ax : z;
  return (a0 == 0.0f) ? (a1 == 0.0f ? 1.0f : 0.0f) : z;
}
static double pow_abs_d(double a0, double a1)
{
  int64_t e;
  const double ax = fabs(a0);
  double x = pow_frexp_d(ax, &e);
  int64_t i = pow_select_d(&x);
  double z = x * x;
  double w = x * (z * horner_d(x, POW1_DP, 4) / horner_d(x, POW1_DQ, 5));
  w = -0.5 * z + w;
  w = db(LOG2_EM1_D) * w + w;
  z = db(LOG2_EM1_D) * x + w;
  z += x;
  w = (double)(-i) * 0.0625 + (double)e;
  const double ya = reduc_d(a1);
  const double yb = a1 - ya;
  double W = z * a1 + w * yb;
  double Wa = reduc_d(W);
  double Wb = W - Wa;
  W = w * ya + Wa;
  Wa = reduc_d(W);
  const double u = W - Wa;
  W = Wb + u;
  Wb = reduc_d(W);
  w = 16.0 * (Wa + Wb);
  const int inf_ret = w > db(POWLARGE_D), zer_ret = w < db(POWLOW_D);
  e = sat_i64(w);
  Wb = W - Wb;
  const int test = Wb > 0.0;
  e = test ? e + 1 : e;
  Wb = Wb - (test ? 0.0625 : 0.0);
  z = horner_d(Wb, POW2_D, 7) * Wb;
  i = (e > 0) ? e / 16 + 1 : e / 16;
  e = i * 16 - e;
  w = db(POW_AD[clamp16(e)]);
  z = w * z + w;
  z = pow_ldexp_d(z, i);
  const int gtax1 = ax > 1.0;
  z = (a1 == INFINITY) ? (gtax1 ? INFINITY : 0.0) : z;
  z = (a1 == -INFINITY) ? (gtax1 ? 0.0 : INFINITY) : z;
  z = (ax == INFINITY) ? (a1 > 0.0 ? INFINITY : (a1 < 0.0 ? 0.0 : 1.0)) : z;
  z = zer_ret ? 0.0 : z;
  z = inf_ret ? INFINITY : z;
  z = (ax == 1.0) ? ax : z;
  return (a0 == 0.0) ? (a1 == 0.0 ? 1.0 : 0.0) : z;
}
/* is_flint(x) = frac(x) == 0 with frac = x - trunc(x) (NaN for Inf/NaN); is_odd(x) =
 * is_flint((x - 1) / 2) (boost/simd/predicates/functions/simd/common/{is_flint,is_even,is_odd}.hpp) */
static inline int is_flint_f(float x) { return isfinite(x) && (x - truncf(x)) == 0.0f; }
static inline int is_flint_d(double x) { return isfinite(x) && (x - trunc(x)) == 0.0; }
EXPORT float nt2o_pow_f(float a0, float a1)
{
  const int ltz = a0 < 0.0f;
  float z = pow_abs_f(a0, a1);
  z = (is_flint_f((a1 - 1.0f) * 0.5f) && ltz) ? -z : z;
  return (ltz && !is_flint_f(a1)) ? NAN : z;
}
EXPORT double nt2o_pow_d(double a0, double a1)
{
  const int ltz = a0 < 0.0;
  double z = pow_abs_d(a0, a1);
  z = (is_flint_d((a1 - 1.0) * 0.5) && ltz) ? -z : z;
  return (ltz && !is_flint_d(a1)) ? NAN : z;
}
EXPORT void nt2o_pow2_f(const float* a0, const float* a1, float* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) y[i] = nt2o_pow_f(a0[i], a1[i]);
}
EXPORT void nt2o_pow2_d(const double* a0, const double* a1, double* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) y[i] = nt2o_pow_d(a0[i], a1[i]);
}

/* --------------------------------------------------- rest of the exp family -- */
/* cbrt, NT2's SIMD forms: exponential/functions/simd/common/cbrt.hpp:36-89 (double, two Newton
 * steps) and :91-142 (float, one), with Boost.SIMD's fast_frexp/fast_ldexp
 * (boost/simd/ieee/functions/simd/common/{fast_frexp,fast_ldexp}.hpp): no special cases inside,
 * zeros and infinities returned as they are at the end. */
static const uint32_t CBRT_PF[5] = {0xbe09e49au, 0x3f0bf0feu, 0xbf745265u, 0x3f91eb77u, 0x3ece0609u};
static const uint64_t CBRT_PD[5] = {0xbfc13c93386fdff6ull, 0x3fe17e1fc7e59d58ull, 0xbfee8a4ca3ba37b8ull,
                                    0x3ff23d6ee505873aull, 0x3fd9c0c12122a4feull};
/* e -> (e / 3 with the sign of e, e mod 3 of |e|) as the integer steps of cbrt.hpp do */
static inline int32_t cbrt_split(int32_t e, int32_t* rem)
{
  int32_t e1 = e < 0 ? -e : e;
  *rem = e1 - (e1 / 3) * 3;
  e1 /= 3;
  return e > 0 ? e1 : (e < 0 ? -e1 : 0);   /* negate(e1, e) = e1 * sign(e) */
}
EXPORT float nt2o_cbrt_f(float a0)
{
  float z = fabsf(a0);
  const int den = z < SMALLESTPOSVAL_F;
  z = den ? z * TWOTONMB_F : z;
  const float f = den ? fb(0x3ba14518u) : 1.0f;          /* Twotomnmbo_3 = 2^(-23/3) */
  const uint32_t b = bf(z);
  int32_t e = (int32_t)((b & 0x7f800000u) >> 23) - 126;
  float x = fb((b & ~0x7f800000u) | 0x3f000000u);
  x = horner_f(x, CBRT_PF, 5);
  const int flag = e >= 0;
  int32_t rem;
  e = cbrt_split(e, &rem);
  float fact = rem == 1 ? (flag ? fb(0x3fa14518u) : fb(0x3f4b2ff5u)) : 1.0f;
  fact = rem == 2 ? (flag ? fb(0x3fcb2ff5u) : fb(0x3f214518u)) : fact;
  x = (x * fact) * fb((uint32_t)(e + 127) << 23);
  x -= (x - z / (x * x)) * fb(0x3eaaaaabu);
  x = fb(bf(x) | (bf(a0) & 0x80000000u)) * f;
  return (a0 == 0.0f || isinf(a0)) ? a0 : x;
}
EXPORT double nt2o_cbrt_d(double a0)
{
  double z = fabs(a0);
  const int den = z < db(0x0010000000000000ull);
  z = den ? z * 4503599627370496.0 : z;
  const double f = den ? db(0x3ed428a2f98d7286ull) : 1.0;  /* 2^(-52/3) */
  const uint64_t b = bd(z);
  int32_t e = (int32_t)((b & 0x7ff0000000000000ull) >> 52) - 1022;
  double x = db((b & ~0x7ff0000000000000ull) | 0x3fe0000000000000ull);
  x = horner_d(x, CBRT_PD, 5);
  const int flag = e >= 0;
  int32_t rem;
  e = cbrt_split(e, &rem);
  double fact = rem == 1 ? (flag ? db(0x3ff428a2f98d728bull) : db(0x3fe965fea53d6e3dull)) : 1.0;
  fact = rem == 2 ? (flag ? db(0x3ff965fea53d6e3dull) : db(0x3fe428a2f98d728bull)) : fact;
  x = (x * fact) * db((uint64_t)(e + 1023) << 52);
  x -= (x - z / (x * x)) * db(0x3fd5555555555555ull);
  x -= (x - z / (x * x)) * db(0x3fd5555555555555ull);
  x = db(bd(x) | (bd(a0) & 0x8000000000000000ull)) * f;
  return (a0 == 0.0 || isinf(a0)) ? a0 : x;
}
/* sqrt1pm1 = sqrt(1+x)-1, generic/sqrt1pm1.hpp:27-33 */
EXPORT float nt2o_sqrt1pm1_f(float a0)
{
  const float t = sqrtf(a0 + 1.0f);
  return fabsf(a0) < 0.5f ? a0 / (t + 1.0f) : t - 1.0f;
}
EXPORT double nt2o_sqrt1pm1_d(double a0)
{
  const double t = sqrt(a0 + 1.0);
  return fabs(a0) < 0.5 ? a0 / (t + 1.0) : t - 1.0;
}
/* exprecneg = exp(-1/x), exprecnegc = -expm1(-1/x): generic/exprecneg.hpp:27, exprecnegc.hpp:27 */
EXPORT float nt2o_exprecneg_f(float a0) { return nt2o_exp_f(-(1.0f / a0)); }
EXPORT double nt2o_exprecneg_d(double a0) { return nt2o_exp_d(-(1.0 / a0)); }
EXPORT float nt2o_exprecnegc_f(float a0) { return -nt2o_expm1_f(-(1.0f / a0)); }
EXPORT double nt2o_exprecnegc_d(double a0) { return -nt2o_expm1_d(-(1.0 / a0)); }
/* expx2(x) = exp(x*x) and expx2(x, s) = exp(sign(s)*x*x) with x*x split at a multiple of
 * 1/Expx2c1: simd/common/expx2.hpp:31-50 and :52-74 (signnz(s): -1 for -0). */
EXPORT float nt2o_expx2s_f(float a0, float s)
{
  const float sgn = (bf(s) & 0x80000000u) ? -1.0f : 1.0f;
  const float x = a0 * sgn;
  const float m = 32.0f * floorf(0.03125f * x + 0.5f);
  const float f = x - m;
  const float u = sgn * (m * m);
  const float u1 = sgn * ((m + m) * f + f * f);
  float r = (u + u1 > MAXLOG_F) ? INFINITY : nt2o_exp_f(u) * nt2o_exp_f(u1);
  return x == INFINITY ? x : r;
}
EXPORT double nt2o_expx2s_d(double a0, double s)
{
  const double sgn = (bd(s) & 0x8000000000000000ull) ? -1.0 : 1.0;
  const double x = a0 * sgn;
  const double m = 128.0 * floor(0.0078125 * x + 0.5);
  const double f = x - m;
  const double u = sgn * (m * m);
  const double u1 = sgn * ((m + m) * f + f * f);
  double r = (u + u1 > MAXLOG_D) ? INFINITY : nt2o_exp_d(u) * nt2o_exp_d(u1);
  return x == INFINITY ? x : r;
}
EXPORT float nt2o_expx2_f(float a0)
{
  const float x = fabsf(a0);
  const float m = 32.0f * floorf(0.03125f * x + 0.5f);
  const float f = x - m;
  const float u = m * m;
  const float u1 = (m + m) * f + f * f;
  float r = (u + u1 > MAXLOG_F) ? INFINITY : nt2o_exp_f(u) * nt2o_exp_f(u1);
  return x == INFINITY ? x : r;
}
EXPORT double nt2o_expx2_d(double a0)
{
  const double x = fabs(a0);
  const double m = 128.0 * floor(0.0078125 * x + 0.5);
  const double f = x - m;
  const double u = m * m;
  const double u1 = (m + m) * f + f * f;
  double r = (u + u1 > MAXLOG_D) ? INFINITY : nt2o_exp_d(u) * nt2o_exp_d(u1);
  return x == INFINITY ? x : r;
}
/* logspace_add(a, b) = log(exp(a) + exp(b)), simd/common/logspace_add.hpp:27-36;
 * logspace_sub(a, b) = log(exp(a) - exp(b)), simd/common/logspace_sub.hpp:27-35 */
EXPORT float nt2o_logspace_add_f(float a0, float a1)
{
  const float t = -fabsf(a0 - a1);
  const float r = (a0 > a1 ? a0 : a1) + nt2o_log1p_f(nt2o_exp_f(t));
  return isnan(t) ? a0 + a1 : r;
}
EXPORT double nt2o_logspace_add_d(double a0, double a1)
{
  const double t = -fabs(a0 - a1);
  const double r = (a0 > a1 ? a0 : a1) + nt2o_log1p_d(nt2o_exp_d(t));
  return isnan(t) ? a0 + a1 : r;
}
EXPORT float nt2o_logspace_sub_f(float a0, float a1)
{
  const float x = a1 - a0;
  const float t = x > -fb(0x3f317218u) ? nt2o_log_f(-nt2o_expm1_f(x)) : nt2o_log1p_f(-nt2o_exp_f(x));
  return a0 + t;
}
EXPORT double nt2o_logspace_sub_d(double a0, double a1)
{
  const double x = a1 - a0;
  const double t = x > -db(0x3fe62e42fefa39efull) ? nt2o_log_d(-nt2o_expm1_d(x)) : nt2o_log1p_d(-nt2o_exp_d(x));
  return a0 + t;
}
/* hypot, Boost.SIMD's SIMD form (boost/simd/arithmetic/functions/simd/common/hypot.hpp:33-49):
 * e = exponent(max(|a0|, |a1|)) (0 for Inf/NaN, -Maxexponent for 0 and denormals, ieee/functions/
 * simd/common/exponent.hpp), clamped to [Minexponent, Maxexponentm1]; ldexp as in pow; Inf where
 * one argument is NaN and the other infinite. */
static float hypot_f(float a0, float a1)
{
  const float r = fabsf(a0), i = fabsf(a1), m = i > r ? i : r;
  int32_t e = isfinite(m) ? (int32_t)((bf(m) & 0x7f800000u) >> 23) - (m != 0.0f ? 127 : 0) : 0;
  e = e < -126 ? -126 : (e > 126 ? 126 : e);
  const float a = pow_ldexp_f(r, -e), b = pow_ldexp_f(i, -e);
  const float res = pow_ldexp_f(sqrtf(a * a + b * b), e);
  return ((isnan(a0) && isinf(a1)) || (isnan(a1) && isinf(a0))) ? INFINITY : res;
}
static double hypot_d(double a0, double a1)
{
  const double r = fabs(a0), i = fabs(a1), m = i > r ? i : r;
  int64_t e = isfinite(m) ? (int64_t)((bd(m) & 0x7ff0000000000000ull) >> 52) - (m != 0.0 ? 1023 : 0) : 0;
  e = e < -1022 ? -1022 : (e > 1022 ? 1022 : e);
  const double a = pow_ldexp_d(r, -e), b = pow_ldexp_d(i, -e);
  const double res = pow_ldexp_d(sqrt(a * a + b * b), e);
  return ((isnan(a0) && isinf(a1)) || (isnan(a1) && isinf(a0))) ? INFINITY : res;
}
/* asinh, NT2's SIMD forms (hyperbolic/functions/simd/common/asinh.hpp:46-64 double, 66-94 float);
 * average(a, b) = a*0.5 + b*0.5; acsch = asinh(rec) (generic/acsch.hpp). */
static const uint32_t ASINH_F[5] = {0x3ca4d6e6u, 0xbd2ee581u, 0x3d9949b1u, 0xbe2aa9adu, 0x3f800000u};
EXPORT float nt2o_asinh_f(float a0)
{
  const float x = fabsf(a0), x2 = x * x;
  const float z = horner_f(x2, ASINH_F, 5) * x;
  const float tmp = x > fb(0x453504f3u) ? x : x * 0.5f + hypot_f(1.0f, x) * 0.5f;
  const float r = x < 0.5f ? z : nt2o_log_f(tmp) + LOG_2_F;
  return fb(bf(r) ^ (bf(a0) & 0x80000000u));
}
EXPORT double nt2o_asinh_d(double a0)
{
  const double x = fabs(a0);
  const int test = x > db(0x4190000000000000ull);
  double z = test ? x - 1.0 : x + (x * x) / (1.0 + hypot_d(1.0, x));
  z = x == INFINITY ? x : z;
  z = nt2o_log1p_d(z) + (test ? LOG_2_D : 0.0);
  return db(bd(z) ^ (bd(a0) & 0x8000000000000000ull));
}
EXPORT float nt2o_pow_abs_f(float a0, float a1) { return pow_abs_f(a0, a1); }
EXPORT double nt2o_pow_abs_d(double a0, double a1) { return pow_abs_d(a0, a1); }

/* Binary maps: op 0 atan2, 1 pow, 2 pow_abs, 3 realpow (= pow), 4 logspace_add, 5 logspace_sub,
 * 6 expx2(a0, a1), 7 atan2d, 8 nbd_atan2, 9 hypot. */
void nt2o_atan2_f(const float* a0, const float* a1, float* y, size_t n);
void nt2o_atan2_d(const double* a0, const double* a1, double* y, size_t n);
void nt2o_atan2x_f(int op, const float* a0, const float* a1, float* y, size_t n);
void nt2o_atan2x_d(int op, const double* a0, const double* a1, double* y, size_t n);
EXPORT int nt2o_map2_f(int op, const float* a0, const float* a1, float* y, size_t n)
{
  if (op == 0) { nt2o_atan2_f(a0, a1, y, n); return 0; }
  if (op == 7 || op == 8) { nt2o_atan2x_f(op - 7, a0, a1, y, n); return 0; }
  for (size_t i = 0; i < n; ++i) {
    switch (op) {
      case 1: case 3: y[i] = nt2o_pow_f(a0[i], a1[i]); break;
      case 2: y[i] = pow_abs_f(a0[i], a1[i]); break;
      case 4: y[i] = nt2o_logspace_add_f(a0[i], a1[i]); break;
      case 5: y[i] = nt2o_logspace_sub_f(a0[i], a1[i]); break;
      case 6: y[i] = nt2o_expx2s_f(a0[i], a1[i]); break;
      case 9: y[i] = hypot_f(a0[i], a1[i]); break;
      default: return 1;
    }
  }
  return 0;
}
EXPORT int nt2o_map2_d(int op, const double* a0, const double* a1, double* y, size_t n)
{
  if (op == 0) { nt2o_atan2_d(a0, a1, y, n); return 0; }
  if (op == 7 || op == 8) { nt2o_atan2x_d(op - 7, a0, a1, y, n); return 0; }
  for (size_t i = 0; i < n; ++i) {
    switch (op) {
      case 1: case 3: y[i] = nt2o_pow_d(a0[i], a1[i]); break;
      case 2: y[i] = pow_abs_d(a0[i], a1[i]); break;
      case 4: y[i] = nt2o_logspace_add_d(a0[i], a1[i]); break;
      case 5: y[i] = nt2o_logspace_sub_d(a0[i], a1[i]); break;
      case 6: y[i] = nt2o_expx2s_d(a0[i], a1[i]); break;
      case 9: y[i] = hypot_d(a0[i], a1[i]); break;
      default: return 1;
    }
  }
  return 0;
}

/* ------------------------------------------------------------- maps ------ */
enum { OP_EXP = 0, OP_LOG = 1, OP_ERFC = 2, OP_NORMCDF = 3, OP_FASTNORMCDF = 4, OP_SQRT = 5,
       OP_ERFC_SCALAR = 6, OP_EXP2 = 7, OP_EXP10 = 8, OP_LOG2 = 9, OP_LOG10 = 10, OP_EXPM1 = 11,
       OP_LOG1P = 12, OP_SINH = 13, OP_COSH = 14, OP_TANH = 15, OP_CBRT = 16, OP_SQRT1PM1 = 17,
       OP_EXPRECNEG = 18, OP_EXPRECNEGC = 19, OP_EXPX2 = 20, OP_ATANH = 21, OP_ACOSH = 22, OP_SECH = 23,
       OP_CSCH = 24, OP_ACOTH = 25, OP_ASECH = 26, OP_ASINH = 27, OP_ACSCH = 28, OP_COTH = 29, OP_SINHC = 30 };

EXPORT int nt2o_map_f(int op, const float* x, float* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) {
    float a = x[i];
    switch (op) {
      case OP_EXP: y[i] = nt2o_exp_f(a); break;
      case OP_LOG: y[i] = nt2o_log_f(a); break;
      case OP_ERFC: y[i] = nt2o_erfc_f(a); break;
      case OP_NORMCDF: y[i] = nt2o_normcdf_f(a); break;
      case OP_FASTNORMCDF: y[i] = nt2o_fastnormcdf_f(a); break;
      case OP_SQRT: y[i] = sqrtf(a); break;
      case OP_ERFC_SCALAR: y[i] = nt2o_erfc_f_scalar(a); break;
      case OP_EXP2: y[i] = nt2o_exp2_f(a); break;
      case OP_EXP10: y[i] = nt2o_exp10_f(a); break;
      case OP_LOG2: y[i] = nt2o_log2_f(a); break;
      case OP_LOG10: y[i] = nt2o_log10_f(a); break;
      case OP_EXPM1: y[i] = nt2o_expm1_f(a); break;
      case OP_LOG1P: y[i] = nt2o_log1p_f(a); break;
      case OP_SINH: y[i] = nt2o_sinh_f(a); break;
      case OP_COSH: y[i] = nt2o_cosh_f(a); break;
      case OP_TANH: y[i] = nt2o_tanh_f(a); break;
      case OP_CBRT: y[i] = nt2o_cbrt_f(a); break;
      case OP_SQRT1PM1: y[i] = nt2o_sqrt1pm1_f(a); break;
      case OP_EXPRECNEG: y[i] = nt2o_exprecneg_f(a); break;
      case OP_EXPRECNEGC: y[i] = nt2o_exprecnegc_f(a); break;
      case OP_EXPX2: y[i] = nt2o_expx2_f(a); break;
      case OP_ATANH: y[i] = nt2o_atanh_f(a); break;
      case OP_ACOSH: y[i] = nt2o_acosh_f(a); break;
      case OP_SECH: y[i] = (float)1 / nt2o_cosh_f(a); break;
      case OP_CSCH: y[i] = (float)1 / nt2o_sinh_f(a); break;
      case OP_ACOTH: y[i] = nt2o_atanh_f((float)1 / a); break;
      case OP_ASECH: y[i] = nt2o_acosh_f((float)1 / a); break;
      case OP_ASINH: y[i] = nt2o_asinh_f(a); break;
      case OP_COTH: y[i] = nt2o_coth_f(a); break;
      case OP_SINHC: y[i] = nt2o_sinhc_f(a); break;
      case OP_ACSCH: y[i] = nt2o_asinh_f((float)1 / a); break;
      default: return 1;
    }
  }
  return 0;
}

EXPORT int nt2o_map_d(int op, const double* x, double* y, size_t n)
{
  for (size_t i = 0; i < n; ++i) {
    double a = x[i];
    switch (op) {
      case OP_EXP: y[i] = nt2o_exp_d(a); break;
      case OP_LOG: y[i] = nt2o_log_d(a); break;
      case OP_ERFC: y[i] = nt2o_erfc_d(a); break;
      case OP_NORMCDF: y[i] = nt2o_normcdf_d(a); break;
      case OP_SQRT: y[i] = sqrt(a); break;
      case OP_ERFC_SCALAR: y[i] = nt2o_erfc_d_scalar(a); break;
      case OP_EXP2: y[i] = nt2o_exp2_d(a); break;
      case OP_EXP10: y[i] = nt2o_exp10_d(a); break;
      case OP_LOG2: y[i] = nt2o_log2_d(a); break;
      case OP_LOG10: y[i] = nt2o_log10_d(a); break;
      case OP_EXPM1: y[i] = nt2o_expm1_d(a); break;
      case OP_LOG1P: y[i] = nt2o_log1p_d(a); break;
      case OP_SINH: y[i] = nt2o_sinh_d(a); break;
      case OP_COSH: y[i] = nt2o_cosh_d(a); break;
      case OP_TANH: y[i] = nt2o_tanh_d(a); break;
      case OP_CBRT: y[i] = nt2o_cbrt_d(a); break;
      case OP_SQRT1PM1: y[i] = nt2o_sqrt1pm1_d(a); break;
      case OP_EXPRECNEG: y[i] = nt2o_exprecneg_d(a); break;
      case OP_EXPRECNEGC: y[i] = nt2o_exprecnegc_d(a); break;
      case OP_EXPX2: y[i] = nt2o_expx2_d(a); break;
      case OP_ATANH: y[i] = nt2o_atanh_d(a); break;
      case OP_ACOSH: y[i] = nt2o_acosh_d(a); break;
      case OP_SECH: y[i] = (double)1 / nt2o_cosh_d(a); break;
      case OP_CSCH: y[i] = (double)1 / nt2o_sinh_d(a); break;
      case OP_ACOTH: y[i] = nt2o_atanh_d((double)1 / a); break;
      case OP_ASECH: y[i] = nt2o_acosh_d((double)1 / a); break;
      case OP_ASINH: y[i] = nt2o_asinh_d(a); break;
      case OP_COTH: y[i] = nt2o_coth_d(a); break;
      case OP_SINHC: y[i] = nt2o_sinhc_d(a); break;
      case OP_ACSCH: y[i] = nt2o_asinh_d((double)1 / a); break;
      default: return 1;
    }
  }
  return 0;
}

/* --------------------------------------------- OpenMP chunking (NT2) ----- */
/* Transform grain = L2 bytes / sizeof(T); the spawner runs only when
 * sz > 8*grain (shared_memory/transform.hpp:38-48); static schedule over
 * chunks of `grain`, the last chunk taking the leftover
 * (openmp/spawner/transform.hpp:47-58).  `threads` <= 0 keeps OpenMP's default. */
static size_t l2_bytes(void)
{
  long v = -1;
#ifdef _SC_LEVEL2_CACHE_SIZE
  v = sysconf(_SC_LEVEL2_CACHE_SIZE);
#endif
  return v > 0 ? (size_t)v : (size_t)1 << 20;
}

EXPORT size_t nt2o_l2_bytes(void) { return l2_bytes(); }

EXPORT int nt2o_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

#ifdef _OPENMP
#define NT2_SPAWN(n, elem_size, threads, ...)                                    \
  do {                                                                           \
    size_t grain_ = l2_bytes() / (elem_size);                                    \
    if (!grain_) grain_ = 1;                                                     \
    if ((n) > 8 * grain_) {                                                      \
      ptrdiff_t nb_ = (ptrdiff_t)((n) / grain_);                                 \
      size_t left_ = (n) % grain_;                                               \
      int th_ = (threads) > 0 ? (threads) : omp_get_max_threads();              \
      _Pragma("omp parallel for schedule(static) num_threads(th_)")              \
      for (ptrdiff_t c_ = 0; c_ < nb_; ++c_) {                                   \
        size_t lo_ = (size_t)c_ * grain_;                                        \
        size_t hi_ = lo_ + ((c_ < nb_ - 1) ? grain_ : grain_ + left_);           \
        for (size_t i = lo_; i < hi_; ++i) { __VA_ARGS__; }                             \
      }                                                                          \
    } else {                                                                     \
      for (size_t i = 0; i < (n); ++i) { __VA_ARGS__; }                                 \
    }                                                                            \
  } while (0)
#else
#define NT2_SPAWN(n, elem_size, threads, ...) \
  do { for (size_t i = 0; i < (n); ++i) { __VA_ARGS__; } } while (0)
#endif

/* ------------------------------------------------------------ configs ---- */
/* saxpy: Y = alpha*X + Y (demo/saxpy/nt2/saxpy_nt2.cpp:39-42).  The proto
 * optimizer rewrites a*b+c to fma (boost/simd/operator/functions/optimize/plus.hpp),
 * which the generic fma evaluates unfused. */
EXPORT void nt2o_saxpy_f(float a, const float* x, float* y, size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(float), threads, y[i] = a * x[i] + y[i]);
}

EXPORT void nt2o_saxpy_d(double a, const double* x, double* y, size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(double), threads, y[i] = a * x[i] + y[i]);
}

/* rgb2grey: gr = 0.3*r + 0.59*g + 0.11*b (demo/rgb2grey/nt2/rgb2grey_nt2.cpp:42-45) */
EXPORT void nt2o_rgb2grey_f(const float* r, const float* g, const float* b, float* gr,
                            size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(float), threads,
            gr[i] = (0.3f * r[i] + 0.59f * g[i]) + 0.11f * b[i]);
}

/* rgb2grey over uint8 planes: the float statement between nt2::cast<float> and
 * nt2::cast<uint8_t> (nt2/operator/functions/container/cast.hpp:133-150; tofloat is
 * exact, touint and group are C conversions, so truncation toward zero on [0, 255]). */
EXPORT void nt2o_rgb2grey_u8(const uint8_t* r, const uint8_t* g, const uint8_t* b, uint8_t* gr,
                             size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(uint8_t), threads,
            gr[i] = (uint8_t)(uint32_t)((0.3f * (float)r[i] + 0.59f * (float)g[i]) + 0.11f * (float)b[i]));
}

/* rgb2yuv: three statements (demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:28-33), each a full pass
 * as NT2 evaluates them:  y = 0.299f*r + 0.587f*g + 0.114f*b;  u = 0.492f*(b - y);
 * v = 0.877f*(r - y). */
EXPORT void nt2o_rgb2yuv_f(const float* r, const float* g, const float* b, float* y, float* u, float* v,
                           size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(float), threads, y[i] = (0.299f * r[i] + 0.587f * g[i]) + 0.114f * b[i]);
  NT2_SPAWN(n, sizeof(float), threads, u[i] = 0.492f * (b[i] - y[i]));
  NT2_SPAWN(n, sizeof(float), threads, v[i] = 0.877f * (r[i] - y[i]));
}

/* linspace(lo, hi, n): step = (hi-lo)/float(n-1); element p is hi at p = n-1, else
 * fma(p, step, lo) with the generic unfused fma
 * (modules/core/generative/include/nt2/core/functions/details/linspace.hpp:27-45). */
EXPORT void nt2o_linspace_f(float lo, float hi, size_t n, float* out)
{
  if (!n) return;
  float step = (hi - lo) / (float)(n - 1);
  for (size_t p = 0; p < n; ++p) out[p] = (p == n - 1) ? hi : (float)p * step + lo;
}

/* The mandelbrot demo's step functor (demo/mandelbrot/nt2/mandelbrot_nt2.cpp:55-81) on
 * one pack of `w` lanes: iterate the whole pack until no lane has |z|^2 < 4 (taken
 * before the update) or 256 trips; each lane counts the trips on which it held. */
static void mandel_pack(const float* a, const float* b, int32_t* out, int w)
{
  float x[32], y[32];
  int32_t it[32];
  for (int l = 0; l < w; ++l) { x[l] = 0.f; y[l] = 0.f; it[l] = 0; }
  for (int i = 0; i < 256; ++i) {
    int any = 0;
    for (int l = 0; l < w; ++l) {
      float x2 = x[l] * x[l];
      float y2 = y[l] * y[l];
      float xy = 2.0f * x[l] * y[l];
      x[l] = x2 - y2 + a[l];
      y[l] = xy + b[l];
      float m2 = x2 + y2;
      int mask = m2 < 4.0f;
      it[l] += mask;
      any |= mask;
    }
    if (!any) break;
  }
  for (int l = 0; l < w; ++l) out[l] = it[l];
}

/* C = arrayfun(step, A, B) with NT2's transform skeleton: packs of `pack` elements
 * from index 0, then the n % pack tail one element at a time
 * (modules/core/base/include/nt2/core/functions/simd/transform.hpp:40-57). */
EXPORT int nt2o_mandelbrot_f(const float* A, const float* B, int32_t* C, size_t n, int pack, int threads)
{
  if (pack < 1 || pack > 32) return -1;
  size_t np = n / (size_t)pack, nfull = np * (size_t)pack;
#ifdef _OPENMP
  int th = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(th)
#endif
  for (ptrdiff_t k = 0; k < (ptrdiff_t)np; ++k)
    mandel_pack(A + (size_t)k * pack, B + (size_t)k * pack, C + (size_t)k * pack, pack);
  for (size_t e = nfull; e < n; ++e) mandel_pack(A + e, B + e, C + e, 1);
  (void)threads;
  return 0;
}

/* The demo's program: A = expand_to(linspace(a0,a1,w),h,w), B = expand_to(colvect(linspace(b0,b1,h)),h,w)
 * (mandelbrot_nt2.cpp:107-108), column-major, then C = arrayfun(step, A, B). */
EXPORT int nt2o_mandelbrot_grid_f(float a0, float a1, float b0, float b1, size_t h, size_t w, int32_t* C,
                                  int pack, int threads)
{
  size_t n = h * w;
  float* la = (float*)malloc((w ? w : 1) * sizeof(float));
  float* lb = (float*)malloc((h ? h : 1) * sizeof(float));
  float* A = (float*)malloc((n ? n : 1) * sizeof(float));
  float* B = (float*)malloc((n ? n : 1) * sizeof(float));
  int rc = -1;
  if (la && lb && A && B) {
    nt2o_linspace_f(a0, a1, w, la);
    nt2o_linspace_f(b0, b1, h, lb);
    for (size_t j = 0; j < w; ++j)
      for (size_t i = 0; i < h; ++i) { A[i + j * h] = la[j]; B[i + j * h] = lb[i]; }
    rc = nt2o_mandelbrot_f(A, B, C, n, pack, threads);
  }
  free(la); free(lb); free(A); free(B);
  return rc;
}

/* Black-Scholes call and put, written as the NT2 table expression
 *   da = sqrt(T); vda = v*da;
 *   d1 = (log(S/K) + fma(sqr(v),0.5,r)*T) / vda;   d2 = d1 - vda;
 *   e  = K*exp(-r*T);
 *   tie(call,put) = tie(fnms(e,cdf(d2),S*cdf(d1)), fnms(S,cdf(-d1),e*cdf(-d2)));
 * cdf = normcdf (cdf_kind 0) or fastnormcdf (cdf_kind 1, float only). */
static inline void bs_one_f(float S, float K, float T, float r, float v, int cdf,
                            float* call, float* put)
{
  float da = sqrtf(T);
  float vda = v * da;
  float d1 = (nt2o_log_f(S / K) + ((v * v) * 0.5f + r) * T) / vda;
  float d2 = d1 - vda;
  float e = K * nt2o_exp_f((-r) * T);
  float n1, n2, m1, m2;
  if (cdf == 0) {
    n1 = nt2o_normcdf_f(d1); n2 = nt2o_normcdf_f(d2);
    m1 = nt2o_normcdf_f(-d1); m2 = nt2o_normcdf_f(-d2);
  } else {
    n1 = nt2o_fastnormcdf_f(d1); n2 = nt2o_fastnormcdf_f(d2);
    m1 = nt2o_fastnormcdf_f(-d1); m2 = nt2o_fastnormcdf_f(-d2);
  }
  *call = S * n1 - e * n2;
  *put = e * m2 - S * m1;
}

EXPORT void nt2o_bs_f(const float* S, const float* K, const float* T, float r, float v,
                      float* call, float* put, size_t n, int cdf, int threads)
{
  NT2_SPAWN(n, sizeof(float), threads, bs_one_f(S[i], K[i], T[i], r, v, cdf, &call[i], &put[i]));
}

static inline void bs_one_d(double S, double K, double T, double r, double v,
                            double* call, double* put)
{
  double da = sqrt(T);
  double vda = v * da;
  double d1 = (nt2o_log_d(S / K) + ((v * v) * 0.5 + r) * T) / vda;
  double d2 = d1 - vda;
  double e = K * nt2o_exp_d((-r) * T);
  *call = S * nt2o_normcdf_d(d1) - e * nt2o_normcdf_d(d2);
  *put = e * nt2o_normcdf_d(-d2) - S * nt2o_normcdf_d(-d1);
}

EXPORT void nt2o_bs_d(const double* S, const double* K, const double* T, double r, double v,
                      double* call, double* put, size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(double), threads, bs_one_d(S[i], K[i], T[i], r, v, &call[i], &put[i]));
}

/* Demo form, verbatim (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59):
 *   da = sqrt(Ta); d1 = log(Sa/Xa) + (fma(sqr(va),0.5,ra)*Ta)/(va*da);
 *   d2 = fnms(va,da,d1); R = fnms(Xa*exp(-ra*Ta), fastnormcdf(d2), Sa*fastnormcdf(d1)); */
EXPORT void nt2o_bs_demo_f(const float* S, const float* X, const float* T, const float* r,
                           const float* v, float* R, size_t n, int threads)
{
  NT2_SPAWN(n, sizeof(float), threads, {
    float da = sqrtf(T[i]);
    float d1 = nt2o_log_f(S[i] / X[i]) + (((v[i] * v[i]) * 0.5f + r[i]) * T[i]) / (v[i] * da);
    float d2 = d1 - v[i] * da;
    R[i] = S[i] * nt2o_fastnormcdf_f(d1) - (X[i] * nt2o_exp_f((-r[i]) * T[i])) * nt2o_fastnormcdf_f(d2);
  });
}

/* sigmadelta, NT2 form (demo/sigmadelta/nt2/sigmadelta_nt2.cpp:37-58) with
 * saturating adds on uint8.  For each pixel of each of `nframes` frames
 * starting at frame `first`: update bkg and var in place, write the label. */
static inline void sd_pixel(uint8_t* bkg, uint8_t fr, uint8_t* var, uint8_t* out)
{
  uint8_t b = *bkg, v = *var;
  b = (b < fr) ? (uint8_t)(b + 1) : ((b > fr) ? (uint8_t)(b - 1) : b);
  uint8_t d = (uint8_t)((b > fr ? b : fr) - (b < fr ? b : fr));
  unsigned s2 = (unsigned)d + d; if (s2 > 255) s2 = 255;
  unsigned s3 = s2 + d; if (s3 > 255) s3 = 255;
  uint8_t m = (uint8_t)s3;
  if (d != 0) v = (v < m) ? (uint8_t)(v + 1) : ((v > m) ? (uint8_t)(v - 1) : v);
  *out = (d < v) ? 0 : 1;
  *bkg = b; *var = v;
}

/* frames: nframes planes of npix bytes, `frame_stride` bytes apart.
 * If init != 0: bkg = frame 0, var = 1, then frames 1..nframes-1 are processed
 * (the demo's setup and loop, sigmadelta_nt2.cpp:85-106); labels gets
 * nframes-1 planes.  Else all nframes frames are processed from the given
 * bkg/var and labels gets nframes planes.  Labels planes are npix apart. */
EXPORT void nt2o_sigmadelta_u8(const uint8_t* frames, size_t frame_stride, size_t npix, int nframes,
                               uint8_t* bkg, uint8_t* var, uint8_t* labels, int init, int threads)
{
  int first = init ? 1 : 0;
  NT2_SPAWN(npix, 1, threads, {
    uint8_t b, v;
    if (init) { b = frames[i]; v = 1; } else { b = bkg[i]; v = var[i]; }
    for (int k = first; k < nframes; ++k)
      sd_pixel(&b, frames[(size_t)k * frame_stride + i], &v, &labels[(size_t)(k - first) * npix + i]);
    bkg[i] = b; var[i] = v;
  });
}

/* -------------------------------------------------------------- folds ---- */
/* Neumaier-compensated double sum of float terms; the FP64 oracle for the
 * FP32 folds. */
typedef struct { double s, c; } nsum_t;
static inline void nadd(nsum_t* a, double x)
{
  double t = a->s + x;
  if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x; else a->c += (x - t) + a->s;
  a->s = t;
}

EXPORT double nt2o_sum_fp64_f(const float* x, size_t n, double* abs_sum)
{
  nsum_t a = {0, 0}, b = {0, 0};
  for (size_t i = 0; i < n; ++i) { nadd(&a, (double)x[i]); nadd(&b, fabs((double)x[i])); }
  if (abs_sum) *abs_sum = b.s + b.c;
  return a.s + a.c;
}

/* sum over i of x[i]*y[i], products exact in double */
EXPORT double nt2o_dot_fp64_f(const float* x, const float* y, size_t n, double* abs_sum)
{
  nsum_t a = {0, 0}, b = {0, 0};
  for (size_t i = 0; i < n; ++i) {
    double p = (double)x[i] * (double)y[i];
    nadd(&a, p); nadd(&b, fabs(p));
  }
  if (abs_sum) *abs_sum = b.s + b.c;
  return a.s + a.c;
}

EXPORT double nt2o_sum_fp64_d(const double* x, size_t n, double* abs_sum)
{
  nsum_t a = {0, 0}, b = {0, 0};
  for (size_t i = 0; i < n; ++i) { nadd(&a, x[i]); nadd(&b, fabs(x[i])); }
  if (abs_sum) *abs_sum = b.s + b.c;
  return a.s + a.c;
}

/* NT2's single-thread FP32 inner fold of one contiguous column: N-lane
 * accumulators over the nb_vec*N body, horizontal sum of the lanes in lane
 * order, then the scalar tail (core/functions/simd/inner_fold.hpp:49-63).
 * `prod` = y != NULL folds x[i]*y[i] (globalsum(X*Y), demo/sdot/nt2/sdot_nt2.cpp:35-38). */
static float fold_nt2_f(const float* x, const float* y, size_t n, int lanes)
{
  float acc[64];
  if (lanes < 1) lanes = 1;
  if (lanes > 64) lanes = 64;
  for (int l = 0; l < lanes; ++l) acc[l] = 0.0f;
  size_t nb = n / (size_t)lanes, body = nb * (size_t)lanes;
  for (size_t v = 0; v < nb; ++v)
    for (int l = 0; l < lanes; ++l) {
      size_t i = v * (size_t)lanes + (size_t)l;
      acc[l] = acc[l] + (y ? x[i] * y[i] : x[i]);
    }
  float s = acc[0];
  for (int l = 1; l < lanes; ++l) s = s + acc[l];
  for (size_t i = body; i < n; ++i) s = s + (y ? x[i] * y[i] : x[i]);
  return s;
}

EXPORT float nt2o_globalsum_nt2_f(const float* x, size_t n, int lanes) { return fold_nt2_f(x, NULL, n, lanes); }
EXPORT float nt2o_dot_nt2_f(const float* x, const float* y, size_t n, int lanes) { return fold_nt2_f(x, y, n, lanes); }

/* Column sums of a column-major rows x cols table (sum(A,1), inner_fold).
 * out32 gets NT2's FP32 lane order, out64 the compensated FP64 sums and
 * abs64 the sums of |a| (for error bounds); any may be NULL. */
EXPORT void nt2o_inner_fold_f(const float* A, size_t rows, size_t cols, int lanes,
                              float* out32, double* out64, double* abs64, int threads)
{
  (void)threads;
#ifdef _OPENMP
  int th = threads > 0 ? threads : omp_get_max_threads();
  #pragma omp parallel for schedule(static) num_threads(th)
#endif
  for (ptrdiff_t j = 0; j < (ptrdiff_t)cols; ++j) {
    const float* c = A + (size_t)j * rows;
    if (out32) out32[j] = fold_nt2_f(c, NULL, rows, lanes);
    if (out64 || abs64) {
      double ab;
      double s = nt2o_sum_fp64_f(c, rows, &ab);
      if (out64) out64[j] = s;
      if (abs64) abs64[j] = ab;
    }
  }
}

/* Row sums of a column-major rows x cols table (sum(A,2), outer_fold): NT2
 * walks the columns in order and accumulates each row
 * (core/functions/details/outer_fold_step.hpp:49-66), so its FP32 result is
 * the plain sequential sum per row. */
EXPORT void nt2o_outer_fold_f(const float* A, size_t rows, size_t cols,
                              float* out32, double* out64, double* abs64, int threads)
{
  (void)threads;
#ifdef _OPENMP
  int th = threads > 0 ? threads : omp_get_max_threads();
  #pragma omp parallel for schedule(static) num_threads(th)
#endif
  for (ptrdiff_t i = 0; i < (ptrdiff_t)rows; ++i) {
    float s = 0.0f;
    nsum_t a = {0, 0}, b = {0, 0};
    for (size_t m = 0; m < cols; ++m) {
      float x = A[m * rows + (size_t)i];
      s = s + x;
      nadd(&a, x); nadd(&b, fabs((double)x));
    }
    if (out32) out32[i] = s;
    if (out64) out64[i] = a.s + a.c;
    if (abs64) abs64[i] = b.s + b.c;
  }
}

/* Timed CPU baseline for the folds: NT2's OpenMP fold spawner splits the
 * vectorised part into blocks of one L2 cache line's worth of elements
 * (shared_memory/worker/inner_fold.hpp:53-56, openmp/spawner/fold.hpp:49-66)
 * and combines the per-block partials in arrival order.  Arrival order is
 * what makes NT2's FP32 sums vary run to run; here the combine is an OpenMP
 * reduction, the same class of order. */
/* Row sums (sum(A,2)) with the loop structure of NT2's shared-memory
 * outer_fold in its in-cache branch (arch/shared_memory/.../worker/outer_fold.hpp:119-147,
 * reduction/.../details/outer_fold_step.hpp:33-66): the rows are cut into
 * chunks of one 64-byte line of floats (16), chunks are spread over the
 * threads by the transform spawner's static schedule (openmp/spawner/transform.hpp:47-58,
 * the last chunk taking the leftover), and each chunk adds the columns one
 * after another into its 16 outputs.  Every output is the sequential FP32 sum
 * over the columns, as out32 of nt2o_outer_fold_f; this form is the one to
 * time. */
EXPORT void nt2o_outer_fold_nt2_f(const float* A, size_t rows, size_t cols, float* out, int threads)
{
  const size_t grain = 16;
  const size_t iib = rows / 4 * 4;
  (void)threads;
  if (iib >= grain) {
    const ptrdiff_t nb = (ptrdiff_t)(iib / grain);
    const size_t left = iib % grain;
#ifdef _OPENMP
    int th = threads > 0 ? threads : omp_get_max_threads();
    #pragma omp parallel for schedule(static) num_threads(th)
#endif
    for (ptrdiff_t c = 0; c < nb; ++c) {
      const size_t lo = (size_t)c * grain, hi = lo + ((c < nb - 1) ? grain : grain + left);
      for (size_t i = lo; i < hi; ++i) out[i] = 0.0f;
      for (size_t m = 0; m < cols; ++m) {
        const float* a = A + m * rows;
        for (size_t i = lo; i < hi; ++i) out[i] = out[i] + a[i];
      }
    }
  }
  for (size_t i = (iib >= grain ? iib : 0); i < rows; ++i) {
    float s = 0.0f;
    for (size_t m = 0; m < cols; ++m) s = s + A[m * rows + i];
    out[i] = s;
  }
}

/* Many sigma-delta streams, each the NT2 statement of nt2o_sigmadelta_u8.
 * NT2 evaluates one stream's statement at a time and runs it on one thread
 * while its table is below the spawner's threshold (8 * L2 bytes of
 * pixels), which every stream of a 1920x1080 or smaller video is; the
 * streams themselves are independent, so this spreads whole streams over
 * the threads (the most a caller of NT2 gets from the host cores). */
EXPORT void nt2o_sigmadelta_batch_u8(int nstreams, const uint8_t* const* frames, const size_t* frame_stride,
                                     const size_t* npix, int nframes, uint8_t* const* bkg, uint8_t* const* var,
                                     uint8_t* const* labels, int init, int threads)
{
  (void)threads;
#ifdef _OPENMP
  int th = threads > 0 ? threads : omp_get_max_threads();
  #pragma omp parallel for schedule(dynamic, 1) num_threads(th)
#endif
  for (int k = 0; k < nstreams; ++k)
    nt2o_sigmadelta_u8(frames[k], frame_stride[k], npix[k], nframes, bkg[k], var[k], labels[k], init, 1);
}

EXPORT float nt2o_dot_omp_f(const float* x, const float* y, size_t n, int lanes, int threads)
{
  (void)lanes;
  float s = 0.0f;
#ifdef _OPENMP
  int th = threads > 0 ? threads : omp_get_max_threads();
  #pragma omp parallel for schedule(static) reduction(+ : s) num_threads(th)
#endif
  for (ptrdiff_t i = 0; i < (ptrdiff_t)n; ++i) s = s + (y ? x[i] * y[i] : x[i]);
  return s;
}
