/*
 * nt2cuda.h -- C ABI of the GB300 (sm_103a) evaluator for NT2 table
 * expressions.
 *
 * NT2 evaluates `table = expression` through compile-time dispatch on a
 * "site" (cpu_ < simd_ < openmp_/tbb_/hpx_ < shared_memory_) and never leaves
 * the CPU.  This library is the device side of a new site: each entry point
 * below is what that site's overloads of transform_, inner_fold_ and
 * outer_fold_ call (or what any other language binds), with plain pointers
 * and sizes only.  Paths in the citations are relative to the NT2 source tree.
 *
 * Conventions
 *   - Table pointers are DEVICE pointers (HBM) unless the name ends in _host.
 *     Tables are dense and column-major, as nt2::table is.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     Calls are stream-ordered and return once the work is enqueued, except
 *     the _host entry points, which return with the results in host memory.
 *   - Every entry point returns an nt2cuda_status; none calls exit() or traps.
 *   - `fused` = 0 evaluates NT2's fma/fnms/Horner steps unfused (bit-exact
 *     with NT2 built without FMA contraction); 1 uses hardware FMA.
 *   - `precision` (Black-Scholes entry points and the server) takes those two
 *     values and 2 = fast: hardware FMA, the special-function unit for exp and
 *     log, and reciprocal division inside erfc (float only; its distance to the
 *     exact results and to FP64 is stated in the tests).
 */
#ifndef NT2CUDA_H_INCLUDED
#define NT2CUDA_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* nt2cuda_stream;

/* precision modes (see the conventions above) */
enum { NT2CUDA_PREC_EXACT = 0, NT2CUDA_PREC_FUSED = 1, NT2CUDA_PREC_FAST = 2 };

/* Status codes.  NT2's OpenMP spawners capture worker exceptions and drop
 * them (modules/arch/openmp/include/nt2/sdk/openmp/spawner/transform.hpp:40-69);
 * here every failure is returned to the caller. */
typedef enum {
  NT2CUDA_OK = 0,
  NT2CUDA_ERR_ARG = 1,        /* bad pointer, size, shape or option       */
  NT2CUDA_ERR_OOM = 2,        /* device or pinned allocation failed       */
  NT2CUDA_ERR_BUDGET = 3,     /* request exceeds the server memory budget */
  NT2CUDA_ERR_LAUNCH = 4,     /* kernel launch failed                     */
  NT2CUDA_ERR_TIMEOUT = 5,    /* a bounded wait ran out                   */
  NT2CUDA_ERR_CUDA = 6,       /* other CUDA runtime error                 */
  NT2CUDA_ERR_NOT_READY = 7,  /* asynchronous result not ready yet        */
  NT2CUDA_ERR_ALIAS = 8,      /* tables of one statement partially overlap */
  NT2CUDA_ERR_STATE = 9       /* object used in the wrong state           */
} nt2cuda_status;

const char* nt2cuda_status_string(int status);
int nt2cuda_version(void);

/* ------------------------------------------------------------ device ---- */
/* Selects the device and creates its context.  Replaces the cuda_ site's
 * implicit setup (modules/arch/cuda/include/nt2/sdk/cuda/cuda.hpp:16-24). */
nt2cuda_status nt2cuda_init(int device);
nt2cuda_status nt2cuda_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes);
nt2cuda_status nt2cuda_last_cuda_error(int* code);
/* No counterpart in the reference.  *count = device allocations the library
 * has made for its per-stream scratch (fold partials and counters, scan
 * flags, batch descriptors) since it was loaded; a call that needs no new
 * scratch leaves it unchanged. */
nt2cuda_status nt2cuda_scratch_allocations(unsigned long long* count);

/* Device-resident table storage.  Replaces cuda_buffer's cudaMalloc /
 * cudaMemcpyAsync members (modules/arch/cuda/include/nt2/sdk/cuda/memory/buffer.hpp:36-242),
 * whose host-to-device constructor copies a fixed 10 elements (:107-112);
 * these copy exactly `bytes`. */
nt2cuda_status nt2cuda_alloc(size_t bytes, void** ptr);
nt2cuda_status nt2cuda_free(void* ptr);
nt2cuda_status nt2cuda_alloc_host(size_t bytes, void** ptr);   /* pinned */
nt2cuda_status nt2cuda_free_host(void* ptr);
nt2cuda_status nt2cuda_memcpy_h2d(void* dst, const void* src, size_t bytes, nt2cuda_stream stream);
nt2cuda_status nt2cuda_memcpy_d2h(void* dst, const void* src, size_t bytes, nt2cuda_stream stream);
nt2cuda_status nt2cuda_memcpy_d2d(void* dst, const void* src, size_t bytes, nt2cuda_stream stream);
nt2cuda_status nt2cuda_stream_create(nt2cuda_stream* stream);
nt2cuda_status nt2cuda_stream_destroy(nt2cuda_stream stream);
nt2cuda_status nt2cuda_stream_sync(nt2cuda_stream stream);

/* ------------------------------------------------- elementwise transform -- */
/* Elementwise functors for nt2cuda_map_*: NT2's exp/log/erfc/normcdf/
 * fastnormcdf/sqrt (modules/core/exponential/include/nt2/exponential/functions/generic/exp.hpp:19-32,
 * generic/log.hpp:20-31, modules/core/euler/include/nt2/euler/functions/simd/common/erfc.hpp:46-123,
 * modules/core/statistics/include/nt2/statistics/functions/generic/normcdf.hpp:28-34,
 * generic/fastnormcdf.hpp:33-55, boost/simd/arithmetic/functions/scalar/sqrt.hpp:21-62)
 * and exp2/exp10/log2/log10/expm1/log1p
 * (modules/core/exponential/include/nt2/exponential/functions/scalar/impl/expo/{f,d}_expo_reduction.hpp,
 * simd/common/impl/logs/{f,d}_log.hpp, details/expm1_kernel.hpp, simd/common/log1p.hpp)
 * and sin/cos/tan/sinpi/cospi
 * (modules/core/trigonometric/include/nt2/trigonometric/functions/generic/{sin,cos,tan,sinpi,cospi}.hpp
 * over scalar/impl/trigo/trig_base.hpp and simd/common/impl/trigo/trig_base.hpp).
 * NT2's SIMD code reduces the arguments of a whole pack with the method it
 * picks for the pack's largest |x|
 * (functions/scalar/impl/trigo/trig_reduction.hpp:46-183), so its results
 * depend on the pack width.  By default each element is reduced on its own,
 * as NT2's scalar code does (NT2 without a SIMD extension, e.g. on aarch64);
 * with NT2CUDA_MAP_SIMD128 each 16-byte pack (4 floats, 2 doubles, from index
 * 0) is reduced together, as NT2 on a 128-bit SIMD extension does, with the
 * n % pack tail scalar (tables not 16-byte aligned: scalar throughout). */
enum {
  NT2CUDA_OP_EXP = 0,
  NT2CUDA_OP_LOG = 1,
  NT2CUDA_OP_ERFC = 2,
  NT2CUDA_OP_NORMCDF = 3,
  NT2CUDA_OP_FASTNORMCDF = 4, /* float only, as in NT2 */
  NT2CUDA_OP_SQRT = 5,
  NT2CUDA_OP_EXP2 = 6,
  NT2CUDA_OP_EXP10 = 7,
  NT2CUDA_OP_LOG2 = 8,
  NT2CUDA_OP_LOG10 = 9,
  NT2CUDA_OP_EXPM1 = 10,
  NT2CUDA_OP_LOG1P = 11,
  NT2CUDA_OP_SIN = 12,
  NT2CUDA_OP_COS = 13,
  NT2CUDA_OP_TAN = 14,
  NT2CUDA_OP_SINPI = 15,
  NT2CUDA_OP_COSPI = 16,
  NT2CUDA_OP_ASIN = 17,       /* NT2's SIMD forms (simd/common/impl/invtrig) */
  NT2CUDA_OP_ACOS = 18,
  NT2CUDA_OP_ATAN = 19,
  NT2CUDA_OP_SINH = 20,       /* modules/core/hyperbolic: simd/common/{sinh,tanh}.hpp, generic/cosh.hpp */
  NT2CUDA_OP_COSH = 21,
  NT2CUDA_OP_TANH = 22,
  NT2CUDA_OP_CBRT = 23,       /* modules/core/exponential: simd/common/cbrt.hpp (SIMD form) */
  NT2CUDA_OP_SQRT1PM1 = 24,   /* generic/sqrt1pm1.hpp: sqrt(1+x)-1 */
  NT2CUDA_OP_EXPRECNEG = 25,  /* generic/exprecneg.hpp: exp(-1/x) */
  NT2CUDA_OP_EXPRECNEGC = 26, /* generic/exprecnegc.hpp: -expm1(-1/x) */
  NT2CUDA_OP_EXPX2 = 27,      /* simd/common/expx2.hpp: exp(x*x) */
  NT2CUDA_OP_REALSQRT = 28,   /* generic/realsqrt.hpp: sqrt (NT2 asserts x >= 0) */
  NT2CUDA_OP_REALLOG = 29,    /* generic/reallog.hpp: log (NT2 asserts x >= 0) */
  /* composed trigonometric functors (modules/core/trigonometric/.../functions/generic/<name>.hpp;
   * asec: simd/common/asec.hpp).  CSC..CSCD follow NT2CUDA_MAP_SIMD128 as sin, cos, sinpi, cospi do. */
  NT2CUDA_OP_CSC = 30,        /* rec(sin(x)) */
  NT2CUDA_OP_SEC = 31,        /* rec(cos(x)) */
  NT2CUDA_OP_CSCPI = 32,      /* rec(sinpi(x)), NaN at nonzero integers */
  NT2CUDA_OP_SECPI = 33,      /* rec(cospi(x)), NaN where 2x is odd */
  NT2CUDA_OP_CSCD = 34,       /* cscpi(x/180) */
  NT2CUDA_OP_INDEG = 35,      /* radians to degrees */
  NT2CUDA_OP_INRAD = 36,      /* degrees to radians */
  NT2CUDA_OP_ACOT = 37,       /* atan(rec(x)) */
  NT2CUDA_OP_ASIND = 38,      /* indeg(asin(x)) */
  NT2CUDA_OP_ACOSD = 39,
  NT2CUDA_OP_ATAND = 40,
  NT2CUDA_OP_ASINPI = 41,     /* asin(x)/pi */
  NT2CUDA_OP_ACOSPI = 42,
  NT2CUDA_OP_ATANPI = 43,
  NT2CUDA_OP_ACSC = 44,       /* asin(rec(x)) */
  NT2CUDA_OP_ACSCD = 45,      /* indeg(acsc(x)) */
  NT2CUDA_OP_ASEC = 46,       /* pi/2 - acsc(x) */
  NT2CUDA_OP_ASECD = 47,      /* indeg(asec(x)) */
  /* cot and the pi- and degree-unit functors (generic/<name>.hpp: trig_base cota/tana with the
   * pi_tag and degree_tag reductions); they follow NT2CUDA_MAP_SIMD128 as sin and cos do. */
  NT2CUDA_OP_COT = 48,
  NT2CUDA_OP_TANPI = 49,      /* tan(pi x), NaN where x - 1/2 is an integer */
  NT2CUDA_OP_COTPI = 50,      /* cot(pi x), NaN at nonzero integers */
  NT2CUDA_OP_SIND = 51,       /* x in degrees */
  NT2CUDA_OP_COSD = 52,
  NT2CUDA_OP_TAND = 53,       /* NaN at odd multiples of 90 */
  NT2CUDA_OP_COTD = 54,       /* NaN at nonzero multiples of 180 */
  NT2CUDA_OP_SECD = 55,       /* rec(cosd(x)), NaN where cosd(x) is 0 */
  /* fast forms (generic/fast_<name>.hpp): no reduction, NaN outside |x| <= pi/4 (radians),
   * 1/4 (half turns) or 45 (degrees) */
  NT2CUDA_OP_FAST_SIN = 56,
  NT2CUDA_OP_FAST_COS = 57,
  NT2CUDA_OP_FAST_TAN = 58,
  NT2CUDA_OP_FAST_COT = 59,
  NT2CUDA_OP_FAST_SINPI = 60,
  NT2CUDA_OP_FAST_COSPI = 61,
  NT2CUDA_OP_FAST_TANPI = 62,
  NT2CUDA_OP_FAST_COTPI = 63,
  NT2CUDA_OP_FAST_SIND = 64,
  NT2CUDA_OP_FAST_COSD = 65,
  NT2CUDA_OP_FAST_TAND = 66,
  NT2CUDA_OP_FAST_COTD = 67,
  NT2CUDA_OP_SINC = 68,       /* sin(x)/x (simd/common/sinc.hpp); follows NT2CUDA_MAP_SIMD128 */
  NT2CUDA_OP_SINCPI = 69,     /* sinpi(x)/(pi x) (simd/common/sincpi.hpp); follows NT2CUDA_MAP_SIMD128 */
  /* modules/core/hyperbolic: simd/common/{atanh,acosh}.hpp, generic/{sech,csch,acoth,asech}.hpp */
  NT2CUDA_OP_ATANH = 70,
  NT2CUDA_OP_ACOSH = 71,
  NT2CUDA_OP_SECH = 72,       /* rec(cosh(x)) */
  NT2CUDA_OP_CSCH = 73,       /* rec(sinh(x)) */
  NT2CUDA_OP_ACOTH = 74,      /* atanh(rec(x)) */
  NT2CUDA_OP_ASECH = 75,      /* acosh(rec(x)) */
  NT2CUDA_OP_ASINH = 76,      /* simd/common/asinh.hpp (double and float forms differ) */
  NT2CUDA_OP_ACSCH = 77,      /* asinh(rec(x)) */
  NT2CUDA_OP_COTH = 78,       /* simd/common/coth.hpp */
  NT2CUDA_OP_SINHC = 79,      /* simd/common/sinhc.hpp: sinh(x)/x */
  NT2CUDA_OP_PROPER_TANPI = 80  /* modules/core/trigonometric/.../simd/common/proper_tanpi.hpp */
};

/* out = atan2(a0, a1) elementwise (NT2's SIMD form,
 * modules/core/trigonometric/include/nt2/trigonometric/functions/simd/common/atan2.hpp:31-52;
 * atan2(+-0, a1 < 0) is +pi, as there).  flags: NT2CUDA_MAP_FUSED or 0. */
nt2cuda_status nt2cuda_atan2_f32(const float* a0, const float* a1, float* out, size_t n, int flags,
                                 nt2cuda_stream stream);
nt2cuda_status nt2cuda_atan2_f64(const double* a0, const double* a1, double* out, size_t n, int flags,
                                 nt2cuda_stream stream);

/* out = pow(a0, a1) elementwise, a1 floating (NT2's SIMD form, the cephes algorithm:
 * modules/core/exponential/include/nt2/exponential/functions/simd/common/pow.hpp:29-37 over
 * simd/common/pow_abs.hpp:72-131; NaN for a0 < 0 with a1 not an integer, pow(0, 0) = 1,
 * pow(1, anything) = 1).  flags: NT2CUDA_MAP_FUSED or 0. */
nt2cuda_status nt2cuda_pow_f32(const float* a0, const float* a1, float* out, size_t n, int flags,
                               nt2cuda_stream stream);
nt2cuda_status nt2cuda_pow_f64(const double* a0, const double* a1, double* out, size_t n, int flags,
                               nt2cuda_stream stream);

/* Forms of nt2cuda_sincos_*: sincos, sincospi, sincosd and their fast forms
 * (modules/core/trigonometric/.../functions/generic/<name>.hpp: trig_base sincosa, which
 * takes one reduction and gives the values sina and cosa give). */
enum {
  NT2CUDA_SINCOS = 0,
  NT2CUDA_SINCOSPI = 1,
  NT2CUDA_SINCOSD = 2,
  NT2CUDA_FAST_SINCOS = 3,
  NT2CUDA_FAST_SINCOSPI = 4,
  NT2CUDA_FAST_SINCOSD = 5,
  NT2CUDA_SINHCOSH = 6        /* tie(s, c) = sinhcosh(x): modules/core/hyperbolic/.../simd/common/sinhcosh.hpp,
                               * the steps of sinh and cosh, so equal to them bit for bit */
};
/* tie(s, c) = sincos(x) (or the form's variant; sinhcosh for NT2CUDA_SINHCOSH) in one pass over x.  flags: NT2CUDA_MAP_FUSED,
 * NT2CUDA_MAP_SIMD128 (the reduction of the three full forms, as for sin and cos). */
nt2cuda_status nt2cuda_sincos_f32(int form, const float* x, float* s, float* c, size_t n, int flags,
                                  nt2cuda_stream stream);
nt2cuda_status nt2cuda_sincos_f64(int form, const double* x, double* s, double* c, size_t n, int flags,
                                  nt2cuda_stream stream);

/* Binary functors of nt2cuda_map2_*, NT2's SIMD forms (paths under
 * modules/core/exponential/include/nt2/exponential/functions/ unless noted). */
enum {
  NT2CUDA_OP2_ATAN2 = 0,        /* as nt2cuda_atan2_* */
  NT2CUDA_OP2_POW = 1,          /* as nt2cuda_pow_* */
  NT2CUDA_OP2_POW_ABS = 2,      /* simd/common/pow_abs.hpp: |a0|^a1 */
  NT2CUDA_OP2_REALPOW = 3,      /* simd/common/realpow.hpp: pow (NT2 asserts a0 >= 0 or a1 integral) */
  NT2CUDA_OP2_LOGSPACE_ADD = 4, /* simd/common/logspace_add.hpp: log(exp(a0) + exp(a1)) */
  NT2CUDA_OP2_LOGSPACE_SUB = 5, /* simd/common/logspace_sub.hpp: log(exp(a0) - exp(a1)) */
  NT2CUDA_OP2_EXPX2 = 6,        /* simd/common/expx2.hpp:52-74: exp(sign(a1) * a0^2) */
  NT2CUDA_OP2_ATAN2D = 7,       /* modules/core/trigonometric/.../generic/atan2d.hpp: indeg(atan2) */
  NT2CUDA_OP2_NBD_ATAN2 = 8,    /* .../simd/common/nbd_atan2.hpp: atan2 without its Inf/NaN cases */
  NT2CUDA_OP2_HYPOT = 9         /* boost/simd/arithmetic/functions/simd/common/hypot.hpp */
};
/* out = op(a0, a1) elementwise.  Replaces `z = nt2::op(x, y)` over two tables of one
 * floating type, evaluated by transform_.  flags: NT2CUDA_MAP_FUSED or 0. */
nt2cuda_status nt2cuda_map2_f32(int op, const float* a0, const float* a1, float* out, size_t n, int flags,
                                nt2cuda_stream stream);
nt2cuda_status nt2cuda_map2_f64(int op, const double* a0, const double* a1, double* out, size_t n, int flags,
                                nt2cuda_stream stream);

/* Flags of nt2cuda_map_*. */
#define NT2CUDA_MAP_FUSED 1     /* hardware FMA (the `fused` convention above) */
#define NT2CUDA_MAP_SIMD128 2   /* trigonometric ops: 128-bit pack reductions  */

/* y = op(x).  Replaces `y = nt2::op(x)` evaluated by transform_
 * (modules/core/base/include/nt2/core/functions/transform.hpp:23-69).
 * `flags`: NT2CUDA_MAP_FUSED | NT2CUDA_MAP_SIMD128 (0 = exact, scalar packs). */
nt2cuda_status nt2cuda_map_f32(int op, const float* x, float* y, size_t n, int flags, nt2cuda_stream stream);
nt2cuda_status nt2cuda_map_f64(int op, const double* x, double* y, size_t n, int flags, nt2cuda_stream stream);

/* Y = alpha*X + Y (demo/saxpy/nt2/saxpy_nt2.cpp:39-42). */
nt2cuda_status nt2cuda_saxpy_f32(float alpha, const float* x, float* y, size_t n, int fused, nt2cuda_stream stream);
nt2cuda_status nt2cuda_saxpy_f64(double alpha, const double* x, double* y, size_t n, int fused, nt2cuda_stream stream);

/* gr = 0.3*r + 0.59*g + 0.11*b (demo/rgb2grey/nt2/rgb2grey_nt2.cpp:42-45). */
nt2cuda_status nt2cuda_rgb2grey_f32(const float* r, const float* g, const float* b, float* gr, size_t n,
                                    int fused, nt2cuda_stream stream);

/* The same statement over uint8 planes, spelled in NT2 as
 *   gr = cast<uint8_t>(0.3f*cast<float>(r) + 0.59f*cast<float>(g) + 0.11f*cast<float>(b))
 * (nt2/operator/functions/container/cast.hpp:133-150: tofloat on the way in, touint and
 * narrowing on the way out, i.e. truncation toward zero; the sum stays in [0, 255]). */
nt2cuda_status nt2cuda_rgb2grey_u8(const uint8_t* r, const uint8_t* g, const uint8_t* b, uint8_t* gr, size_t n,
                                   int fused, nt2cuda_stream stream);

/* The rgb2yuv demo's three statements (demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:28-33)
 *   y = 0.299f*r + 0.587f*g + 0.114f*b;  u = 0.492f*(b - y);  v = 0.877f*(r - y);
 * in one pass: u and v use the y value the first statement stores, so the
 * result is the one of the three NT2 passes.  The outputs may not overlap the
 * inputs or each other (NT2CUDA_ERR_ALIAS). */
nt2cuda_status nt2cuda_rgb2yuv_f32(const float* r, const float* g, const float* b, float* y, float* u, float* v,
                                   size_t n, int fused, nt2cuda_stream stream);

/* C = arrayfun(step, A, B) of the mandelbrot demo (demo/mandelbrot/nt2/mandelbrot_nt2.cpp:41-83,120-123):
 * per element the escape-time loop z <- z^2 + (a + ib) from z = 0, at most 256
 * trips, counting the trips on which |z|^2 < 4 held before the update.  NT2
 * runs the functor on SIMD packs: a pack keeps iterating while any of its
 * lanes has not escaped, and elements past the last whole pack run alone.
 * `pack` is that cardinality (1, 2, 4, 8, 16 or 32; 8 is AVX float, 1 the
 * scalar build); it changes results only where an escaped orbit re-enters
 * the disc.  Element i of C is an int32 count. */
nt2cuda_status nt2cuda_mandelbrot_f32(const float* A, const float* B, int32_t* C, size_t n, int pack,
                                      nt2cuda_stream stream);
/* The demo's complete program: A = expand_to(linspace(a0,a1,w),h,w) and
 * B = expand_to(colvect(linspace(b0,b1,h)),h,w) generated in the kernel (no
 * input tables; linspace as nt2/core/functions/details/linspace.hpp:33-45), then
 * C (h x w, column-major) = arrayfun(step, A, B).  NT2 accepts the demo's
 * expand_to only for h == w; other shapes follow the same formulas. */
nt2cuda_status nt2cuda_mandelbrot_grid_f32(float a0, float a1, float b0, float b1, size_t h, size_t w,
                                           int32_t* C, int pack, nt2cuda_stream stream);

/* Black-Scholes call and put over n options with scalar rate r and
 * volatility sigma, as the NT2 statement
 *   tie(call,put) = tie(fnms(e,cdf(d2),S*cdf(d1)), fnms(S,cdf(-d1),e*cdf(-d2)))
 *   with d1 = (log(S/K) + fma(sqr(sigma),0.5,r)*T)/(sigma*sqrt(T)),
 *        d2 = d1 - sigma*sqrt(T), e = K*exp(-r*T)
 * in one pass (a tie() assignment, modules/core/container/table/include/nt2/core/functions/expr/tie.hpp:40-74).
 * cdf_kind 0 = normcdf via erfc, 1 = fastnormcdf (float only). */
nt2cuda_status nt2cuda_blackscholes_f32(const float* S, const float* K, const float* T, float r, float sigma,
                                        float* call, float* put, size_t n, int cdf_kind, int precision,
                                        nt2cuda_stream stream);
nt2cuda_status nt2cuda_blackscholes_f64(const double* S, const double* K, const double* T, double r,
                                        double sigma, double* call, double* put, size_t n, int precision,
                                        nt2cuda_stream stream);

/* The Black-Scholes demo statement, verbatim
 * (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59): five input tables,
 * one output R = fnms(X*exp(-r*T), fastnormcdf(d2), S*fastnormcdf(d1)),
 * d1 = log(S/X) + (fma(sqr(v),0.5,r)*T)/(v*sqrt(T)), d2 = fnms(v, sqrt(T), d1). */
nt2cuda_status nt2cuda_blackscholes_demo_f32(const float* S, const float* X, const float* T, const float* r,
                                             const float* v, float* R, size_t n, int fused,
                                             nt2cuda_stream stream);

/* Host-buffer form of nt2cuda_blackscholes_f32 for NT2 tables that live in
 * host memory: copies in, evaluates and copies out in pipelined chunks on
 * library-owned streams and device staging, and returns when call/put hold
 * the results.  Host buffers should be pinned for full copy bandwidth. */
nt2cuda_status nt2cuda_blackscholes_f32_host(const float* S, const float* K, const float* T, float r,
                                             float sigma, float* call, float* put, size_t n, int cdf_kind,
                                             int precision);

/* ------------------------------------------------------------- folds ---- */
/* globalsum(X) and globalsum(X*Y) (modules/core/reduction/include/nt2/core/functions/globalsum.hpp:75-88,
 * demo/sdot/nt2/sdot_nt2.cpp:35-38): the inner_fold over one column of n
 * elements.  *out is a DEVICE scalar.  compensated = 1 accumulates FP32 with
 * TwoSum-compensated partials; 0 is the plain tree sum.  The block
 * decomposition depends only on n, so results are bitwise reproducible.
 * The first call on a stream allocates that stream's scratch. */
nt2cuda_status nt2cuda_globalsum_f32(const float* x, size_t n, float* out, int compensated, nt2cuda_stream stream);
nt2cuda_status nt2cuda_dot_f32(const float* x, const float* y, size_t n, float* out, int compensated,
                               nt2cuda_stream stream);
/* No counterpart in the reference: NT2 has no device code.  globalsum(X*Y)
 * for callers that cannot allocate device memory (their device memory
 * belongs to another allocator, or cudaMalloc's device-wide synchronisation
 * is not acceptable in their loop).  It allocates nothing: its scratch is a
 * fixed 512.25 KiB array in device memory, held by every GPU that loads the
 * library until the process exits.  The result is within nt2cuda_dot_f32's
 * error bound and bitwise reproducible from call to call of this entry point,
 * but it is not bit for bit nt2cuda_dot_f32's (that one takes the TMA fold
 * for long aligned vectors).  n may not exceed NT2CUDA_DOT_NOALLOC_MAX_N
 * (larger n returns NT2CUDA_ERR_ARG).  The first call on a device, and the
 * first after its context was reset, looks up the array's address in that
 * context; make that first call before any stream capture.  All calls share
 * the array, so calls whose kernels overlap on the GPU (other streams, other
 * threads) race; calls on one stream are safe.  *out is a DEVICE scalar. */
#define NT2CUDA_DOT_NOALLOC_MAX_N ((size_t)1 << 30)
nt2cuda_status nt2cuda_dot_f32_noalloc(const float* x, const float* y, size_t n, float* out, int compensated,
                                       nt2cuda_stream stream);
nt2cuda_status nt2cuda_globalsum_f64(const double* x, size_t n, double* out, nt2cuda_stream stream);
nt2cuda_status nt2cuda_dot_f64(const double* x, const double* y, size_t n, double* out, nt2cuda_stream stream);

/* sum(A,1): column sums of a rows x cols column-major table -> out[cols]
 * (inner_fold, modules/core/reduction/include/nt2/core/functions/inner_fold.hpp:21-58,
 *  modules/arch/shared_memory/include/nt2/core/functions/shared_memory/inner_fold.hpp:24-63). */
nt2cuda_status nt2cuda_sum_inner_f32(const float* A, size_t rows, size_t cols, float* out, int compensated,
                                     nt2cuda_stream stream);
nt2cuda_status nt2cuda_sum_inner_f64(const double* A, size_t rows, size_t cols, double* out,
                                     nt2cuda_stream stream);
/* sum(A,2): row sums -> out[rows] (outer_fold,
 * modules/core/reduction/include/nt2/core/functions/outer_fold.hpp:17-55,
 * modules/arch/shared_memory/include/nt2/core/functions/shared_memory/outer_fold.hpp:22-51). */
nt2cuda_status nt2cuda_sum_outer_f32(const float* A, size_t rows, size_t cols, float* out, int compensated,
                                     nt2cuda_stream stream);
nt2cuda_status nt2cuda_sum_outer_f64(const double* A, size_t rows, size_t cols, double* out,
                                     nt2cuda_stream stream);

/* Kernel family for the folds: 0 = automatic (TMA-staged tiles for long
 * columns, register-pipelined kernels otherwise), 1 = register-pipelined
 * only, 2 = TMA-staged wherever the tables allow it.  Results of every family
 * are within the same bounds; each family is bitwise reproducible.  Process-wide. */
nt2cuda_status nt2cuda_set_fold_path(int path);

/* ------------------------------------------------------- reductions ---- */
/* The reductions of NT2's reduction module on the fold kernels, along
 * dim 1 (one value per column: inner_fold, out has cols entries), dim 2
 * (one value per row: outer_fold, out has rows entries) or dim 0 (the whole
 * table, NT2's global* functions: out has 1 entry).
 * (modules/core/reduction/include/nt2/core/functions/expr/{asum1,asum2,norm2,mean,var,stdev}.hpp,
 *  modules/boost/simd/base/include/boost/simd/reduction/functions/{sum,maximum,minimum,prod}.hpp)
 * FP32 sums accumulate compensated unless NT2CUDA_RED_PLAIN is set; var and
 * stdev normalise by n - 1 (NT2's w = 0; by n with NT2CUDA_RED_VAR_N) and are
 * computed in one pass (Welford updates, Chan merges).  max and min skip NaNs;
 * a fold of zero elements gives NT2's neutral value (0, 1, -FLT_MAX, FLT_MAX). */
enum {
  NT2CUDA_RED_SUM = 0, NT2CUDA_RED_ASUM1 = 1, NT2CUDA_RED_ASUM2 = 2, NT2CUDA_RED_NORM2 = 3,
  NT2CUDA_RED_MEAN = 4, NT2CUDA_RED_VAR = 5, NT2CUDA_RED_STDEV = 6, NT2CUDA_RED_MAX = 7,
  NT2CUDA_RED_MIN = 8, NT2CUDA_RED_PROD = 9
};
enum { NT2CUDA_RED_PLAIN = 1, NT2CUDA_RED_VAR_N = 2 };   /* flags */
/* logical reductions: all(A != 0), any(A != 0), none = !any; uint8_t 0/1 outputs
 * (boost/simd/reduction/functions/{all,any,none}.hpp) */
enum { NT2CUDA_RED_ALL = 0, NT2CUDA_RED_ANY = 1, NT2CUDA_RED_NONE = 2 };

nt2cuda_status nt2cuda_reduce_f32(int op, const float* A, size_t rows, size_t cols, int dim, float* out, int flags,
                                  nt2cuda_stream stream);
nt2cuda_status nt2cuda_reduce_f64(int op, const double* A, size_t rows, size_t cols, int dim, double* out,
                                  int flags, nt2cuda_stream stream);
nt2cuda_status nt2cuda_reduce_logical_f32(int op, const float* A, size_t rows, size_t cols, int dim, uint8_t* out,
                                          nt2cuda_stream stream);
nt2cuda_status nt2cuda_reduce_logical_f64(int op, const double* A, size_t rows, size_t cols, int dim, uint8_t* out,
                                          nt2cuda_stream stream);

/* ------------------------------------------------------------- scans ---- */
/* cumsum, cumprod, cummax, cummin of a rows x cols column-major table along
 * dim 1 (down each column: inner_scan) or dim 2 (along each row: outer_scan)
 * (modules/core/swar/include/nt2/dsl/functions/cumulative/run.hpp:27-75,
 *  modules/boost/simd/base/include/boost/simd/swar/functions/{cumsum,cumprod,cummax,cummin}.hpp).
 * out may be A itself (in place) but no other overlap.  FP32 cumsum carries
 * compensated partial sums unless NT2CUDA_RED_PLAIN is set; cummax and cummin
 * skip NaNs.  Results are bitwise reproducible from run to run. */
enum { NT2CUDA_SCAN_SUM = 0, NT2CUDA_SCAN_PROD = 1, NT2CUDA_SCAN_MAX = 2, NT2CUDA_SCAN_MIN = 3 };
nt2cuda_status nt2cuda_scan_f32(int op, const float* A, size_t rows, size_t cols, int dim, float* out, int flags,
                                nt2cuda_stream stream);
nt2cuda_status nt2cuda_scan_f64(int op, const double* A, size_t rows, size_t cols, int dim, double* out, int flags,
                                nt2cuda_stream stream);

/* Scans of columns longer than one tile chain their tiles through bounded
 * waits on each other's published prefixes, and the TMA folds wait (bounded)
 * for their own bulk copies.  A wait that runs out (it means a fault) makes
 * its tile or its fold's column write NaN and is counted: *count = waits that
 * ran out since the library was loaded, over both kinds (synchronous). */
nt2cuda_status nt2cuda_wait_timeouts(unsigned long long* count);
/* Check that a wait which cannot be satisfied runs out and is reported: scans
 * a two-tile column whose first tile no block takes.  Returns
 * NT2CUDA_ERR_TIMEOUT when the kernel reported the timeout (the expected
 * result, after about a second), NT2CUDA_OK if it did not. */
nt2cuda_status nt2cuda_selftest_wait_timeout(nt2cuda_stream stream);
/* The same for the TMA column fold: out = sum(A,1) of a 16-byte aligned
 * rows x cols table (rows a multiple of 4 and above 65536, so every column is
 * split into several units) with the first tile of unit 0 armed but never
 * copied.  That block's wait runs out after a short bound; column 0 becomes
 * NaN, the other columns are the normal result, and the column's arrival
 * counter is left at zero for the next fold on the stream.  Synchronous;
 * returns NT2CUDA_ERR_TIMEOUT when the timeout was reported. */
nt2cuda_status nt2cuda_selftest_fold_timeout(const float* A, size_t rows, size_t cols, float* out,
                                             nt2cuda_stream stream);

/* No counterpart in the reference.  The FP32 Black-Scholes kernels (exact,
 * fused and fast modes) price two options at a time on the packed FP32
 * instructions; this checks their two-lane functors against the one-lane ones
 * over every float argument (2^32 values): which = 0 exp, 1 log, 2 erfc of
 * |a|, 3 normcdf(a) with normcdf(-a); 4..7 the same functors with each NT2
 * fma/fnms one hardware FMA (the fused precision mode); 8..11 the fast mode's
 * exp of a moderate argument, log, erfc of |a| and normcdf pair; 12, 13
 * fastnormcdf(a) with fastnormcdf(-a), unfused and fused; 14..21 the packed
 * evaluation of the float trigonometric functors (sin, cos, then the same
 * fused; tan, cot, then the same fused) over every reduced argument;
 * 22..25 pow, pow fused, pow_abs, pow_abs fused, with every float once as the
 * base and once as the exponent, each against a drawn partner; 26, 27 cbrt,
 * unfused and fused.
 * *mismatches = arguments whose results differ in any bit (two NaNs are
 * equal); first_bad (8 entries, may be NULL) gets the first ones' bit
 * patterns.  Synchronous. */
nt2cuda_status nt2cuda_selftest_x2(int which, unsigned long long* mismatches, uint32_t* first_bad,
                                   nt2cuda_stream stream);

/* --------------------------------------------------------- sigmadelta ---- */
/* One grey video stream for the batched sigma-delta background subtraction
 * (demo/sigmadelta/nt2/sigmadelta_nt2.cpp:37-58, 85-106).  frames holds
 * nframes planes of width*height uint8 pixels, frame_stride bytes apart;
 * labels receives one plane per processed frame, label_stride bytes apart;
 * bkg and var (width*height each) are the background and variance state. */
typedef struct {
  const uint8_t* frames;
  size_t frame_stride;
  uint8_t* bkg;
  uint8_t* var;
  uint8_t* labels;
  size_t label_stride;
  uint32_t width;
  uint32_t height;
} nt2cuda_sd_stream;

/* Process nframes frames of every stream in one persistent launch over a
 * (stream, tile) work-list.  init = 1: bkg = frame 0, var = 1, then frames
 * 1..nframes-1 are processed (nframes-1 label planes); init = 0: all nframes
 * frames are processed from the given bkg/var.  `streams` is a HOST array. */
nt2cuda_status nt2cuda_sigmadelta_batch_u8(const nt2cuda_sd_stream* streams, int nstreams, int nframes, int init,
                                           nt2cuda_stream stream);

/* The same work captured once in a CUDA graph and replayed. */
typedef struct nt2cuda_sd_plan nt2cuda_sd_plan;
nt2cuda_status nt2cuda_sigmadelta_plan_create(const nt2cuda_sd_stream* streams, int nstreams, int nframes, int init,
                                              nt2cuda_stream stream, nt2cuda_sd_plan** plan);
nt2cuda_status nt2cuda_sigmadelta_plan_launch(nt2cuda_sd_plan* plan, nt2cuda_stream stream);
nt2cuda_status nt2cuda_sigmadelta_plan_destroy(nt2cuda_sd_plan* plan);

/* ----------------------------------------------------------- serving ---- */
/* Continuous-batching request server for Black-Scholes pricing requests.
 * NT2 has no counterpart: it evaluates one synchronous statement at a time
 * on the calling thread (modules/core/sdk/include/nt2/core/container/dsl/expression.hpp:161-191).
 * Requests carry DEVICE input tables (which must stay valid until the request
 * completes); outputs are written to server-owned device slots admitted
 * against budget_bytes and stay resident until nt2cuda_server_release.
 * coalesce = 1 launches every admitted request of a step in one kernel over a
 * (request, tile) work-list; 0 launches one kernel per request.  At most
 * max_inflight_batches launches are on the device at once.  coalesce = 2
 * keeps one kernel on the device that drains a ring of requests published in
 * pinned host memory: requests that arrive while it runs join it without a
 * launch; it leaves after 20 ms without requests (every wait it makes is
 * bounded in time) and is launched again by the next request. */
typedef struct {
  size_t budget_bytes;        /* device memory for request outputs          */
  int max_batch_requests;     /* requests coalesced into one launch         */
  int max_inflight_batches;   /* launches on the device at once (streams)   */
  int coalesce;               /* 2 = resident kernel, 1 = batched work-list,
                                 0 = launch per request                     */
  int fused;                  /* precision mode: 0 exact, 1 fused, 2 fast   */
  int cdf_kind;               /* 0 = normcdf, 1 = fastnormcdf               */
  int wait_timeout_ms;        /* default bound of waits (<= 0: 60000)       */
  int spin_us;                /* the launch thread polls this long for new
                                 requests before it sleeps (< 0: 0; 0: 50)   */
} nt2cuda_server_config;

typedef struct {
  uint64_t submitted, completed, batches, launches, options;
  size_t reserved_bytes, peak_reserved_bytes;
  uint64_t admission_waits;   /* submissions that could not be admitted at once */
} nt2cuda_server_stats;

typedef struct nt2cuda_server nt2cuda_server;

nt2cuda_status nt2cuda_server_create(const nt2cuda_server_config* cfg, nt2cuda_server** server);
nt2cuda_status nt2cuda_server_destroy(nt2cuda_server* server);
/* Enqueue one request; never blocks.  Returns NT2CUDA_ERR_BUDGET if the
 * request alone exceeds the budget.  The ticket identifies the request. */
nt2cuda_status nt2cuda_server_submit(nt2cuda_server* server, const float* S, const float* K, const float* T, float r,
                                     float sigma, size_t n, uint64_t* ticket);
/* NT2CUDA_OK with the device output pointers once done, else NT2CUDA_ERR_NOT_READY. */
nt2cuda_status nt2cuda_server_poll(nt2cuda_server* server, uint64_t ticket, float** call, float** put);
/* Bounded wait (timeout_ms < 0: the configured default); NT2CUDA_ERR_TIMEOUT when it runs out. */
nt2cuda_status nt2cuda_server_wait(nt2cuda_server* server, uint64_t ticket, int timeout_ms, float** call,
                                   float** put);
/* Return a finished request's output slots to the budget. */
nt2cuda_status nt2cuda_server_release(nt2cuda_server* server, uint64_t ticket);
/* Submit-to-completion latency of a finished request. */
nt2cuda_status nt2cuda_server_latency_ns(nt2cuda_server* server, uint64_t ticket, uint64_t* ns);
nt2cuda_status nt2cuda_server_drain(nt2cuda_server* server, int timeout_ms);
nt2cuda_status nt2cuda_server_get_stats(nt2cuda_server* server, nt2cuda_server_stats* stats);
/* Open-loop replay of a request trace, driven natively: request i (inputs
 * S/K/T + offsets[i] elements, sizes[i] options) is submitted arrival_ns[i]
 * after the call starts; a collector thread waits for the requests in
 * submission order, stores each one's submit-to-completion latency in
 * latency_ns[i] and releases it at once.  Returns when every request is
 * released, or with the first failing status; *elapsed_ns is the time from
 * the start to the last completion.  Measures the server without a client's
 * own overheads (capacity planning, the serving benchmark). */
nt2cuda_status nt2cuda_server_replay(nt2cuda_server* server, const float* S, const float* K, const float* T,
                                     float r, float sigma, size_t nreq, const uint64_t* offsets,
                                     const uint64_t* sizes, const uint64_t* arrival_ns, uint64_t* latency_ns,
                                     uint64_t* elapsed_ns);

/* ------------------------------------------------------------ tuning ---- */
/* Times the launch variants of one entry point at size n on scratch tables
 * and records the fastest for n's size bucket.  kernel: "saxpy_f32",
 * "saxpy_f64", "bs_f32", "bs_f32_fused", "bs_f32_fast", "bs_f64",
 * "bs_f64_fused" (the Black-Scholes keys are per precision mode), and
 * "bs_f32_mapped", "bs_f32_fast_mapped" (the kernel on pinned host tables,
 * as nt2cuda_blackscholes_f32_host runs it), "rgb2grey_u8". */
nt2cuda_status nt2cuda_autotune(const char* kernel, size_t n, int* best_unroll, int* best_waves, float* best_ms);
/* Tuning table as text ("key@bucket unroll waves" lines). */
nt2cuda_status nt2cuda_tuning_export(char* buf, size_t cap, size_t* needed);
nt2cuda_status nt2cuda_tuning_import(const char* text, int* entries);

/* ---------------------------------------------------- synthetic inputs ---- */
/* Seeded counter-based generators (SplitMix64 of seed and element index),
 * so a table's contents depend only on (seed, index). */
nt2cuda_status nt2cuda_fill_uniform_f32(float* x, size_t n, float lo, float hi, uint64_t seed, nt2cuda_stream stream);
nt2cuda_status nt2cuda_fill_uniform_f64(double* x, size_t n, double lo, double hi, uint64_t seed,
                                        nt2cuda_stream stream);
nt2cuda_status nt2cuda_fill_normal_f32(float* x, size_t n, uint64_t seed, nt2cuda_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* NT2CUDA_H_INCLUDED */
