// capi_transform.cu -- C-ABI entry points for elementwise statements: the
// NT2 transform_ site overload lowered for the demo and benchmark statements.
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "internal.cuh"
#include "nt2cuda/blackscholes.cuh"
#include "nt2cuda/expr.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;

namespace {

template <class T, class E> inline assign<T, E> asg(T* out, E e) { return assign<T, E>{out, e}; }
template <class T> inline term<T> tm(const T* p) { return term<T>{p}; }
template <class T> inline scal<T> sc(T v) { return scal<T>{v}; }
template <class Tag, class... C> inline node<Tag, C...> nd(C... c) { return node<Tag, C...>{c...}; }

template <bool F, class P> nt2cuda_status run(const P& p, size_t n, nt2cuda_stream s, const char* key)
{
  return launch_status(transform<F>(p, n, as_stream(s), key));
}

template <bool F, class T> nt2cuda_status map_impl(int op, const T* x, T* y, size_t n, nt2cuda_stream s)
{
  auto X = tm(x);
  switch (op) {
    case NT2CUDA_OP_EXP: return run<F>(make_prog(asg(y, nd<tag::exp_>(X))), n, s, "map");
    case NT2CUDA_OP_LOG: return run<F>(make_prog(asg(y, nd<tag::log_>(X))), n, s, "map");
    case NT2CUDA_OP_ERFC: return run<F>(make_prog(asg(y, nd<tag::erfc_>(X))), n, s, "map");
    case NT2CUDA_OP_NORMCDF: return run<F>(make_prog(asg(y, nd<tag::normcdf_>(X))), n, s, "map");
    case NT2CUDA_OP_SQRT: return run<F>(make_prog(asg(y, nd<tag::sqrt_>(X))), n, s, "map");
    case NT2CUDA_OP_EXP2: return run<F>(make_prog(asg(y, nd<tag::exp2_>(X))), n, s, "map");
    case NT2CUDA_OP_EXP10: return run<F>(make_prog(asg(y, nd<tag::exp10_>(X))), n, s, "map");
    case NT2CUDA_OP_LOG2: return run<F>(make_prog(asg(y, nd<tag::log2_>(X))), n, s, "map");
    case NT2CUDA_OP_LOG10: return run<F>(make_prog(asg(y, nd<tag::log10_>(X))), n, s, "map");
    case NT2CUDA_OP_EXPM1: return run<F>(make_prog(asg(y, nd<tag::expm1_>(X))), n, s, "map");
    case NT2CUDA_OP_LOG1P: return run<F>(make_prog(asg(y, nd<tag::log1p_>(X))), n, s, "map");
    case NT2CUDA_OP_FASTNORMCDF:
      if constexpr (sizeof(T) == 4) return run<F>(make_prog(asg(y, nd<tag::fastnormcdf_>(X))), n, s, "map");
      else return NT2CUDA_ERR_ARG;
    default: return NT2CUDA_ERR_ARG;
  }
}

// Y = alpha*X + Y; the proto optimizer turns a*b+c into fma(a,b,c)
// (boost/simd/operator/functions/optimize/plus.hpp:20-45).
template <bool F, class T> nt2cuda_status saxpy_impl(T a, const T* x, T* y, size_t n, nt2cuda_stream s)
{
  return run<F>(make_prog(asg(y, nd<tag::fma_>(sc(a), tm(x), tm((const T*)y)))), n, s,
                sizeof(T) == 4 ? "saxpy_f32" : "saxpy_f64");
}

// gr = T(0.3)*r + T(0.59)*g + T(0.11)*b  ->  fma(0.11, b, fma(0.3, r, 0.59*g))
template <bool F> nt2cuda_status rgb2grey_impl(const float* r, const float* g, const float* b, float* gr,
                                               size_t n, nt2cuda_stream s)
{
  auto e = nd<tag::fma_>(sc(0.11f), tm(b),
                         nd<tag::fma_>(sc(0.3f), tm(r), nd<tag::multiplies_>(sc(0.59f), tm(g))));
  return run<F>(make_prog(asg(gr, e)), n, s, "rgb2grey");
}

// gr = cast<uint8_t>(T(0.3)*cast<float>(r) + T(0.59)*cast<float>(g) + T(0.11)*cast<float>(b)),
// the float statement's tree between the two casts.
template <bool F> nt2cuda_status rgb2grey_u8_impl(const uint8_t* r, const uint8_t* g, const uint8_t* b,
                                                  uint8_t* gr, size_t n, nt2cuda_stream s)
{
  auto fr = nd<tag::cast_>(tm(r), sc(0.0f));
  auto fg = nd<tag::cast_>(tm(g), sc(0.0f));
  auto fb = nd<tag::cast_>(tm(b), sc(0.0f));
  auto e = nd<tag::fma_>(sc(0.11f), fb, nd<tag::fma_>(sc(0.3f), fr, nd<tag::multiplies_>(sc(0.59f), fg)));
  // 0.3f + 0.59f + 0.11f < 1 and every term is >= 0, so the sum stays in [0, 255]
  return run<F>(make_prog(asg(gr, nd<tag::trunc_u8_>(e))), n, s, "rgb2grey_u8");
}

// rgb2yuv: the three statements of one pixel, with u and v reading the y that
// the first statement stores (the proto optimizer gives y the tree
// fma(0.114, b, fma(0.299, r, 0.587*g)), as for rgb2grey).
template <bool F> struct yuv {
  __device__ __forceinline__ static void px(float r, float g, float b, float& y, float& u, float& v)
  {
    y = math::madd<F>(0.114f, b, math::madd<F>(0.299f, r, math::mul(0.587f, g)));
    u = math::mul(0.492f, math::sub(b, y));
    v = math::mul(0.877f, math::sub(r, y));
  }
};

template <bool F>
__global__ void __launch_bounds__(256) k_rgb2yuv(const float* __restrict__ r, const float* __restrict__ g,
                                                 const float* __restrict__ b, float* __restrict__ y,
                                                 float* __restrict__ u, float* __restrict__ v, size_t n)
{
  nt2cuda::mem::pdl_begin();
  constexpr int V = 4;
  const size_t groups = n / V;
  const size_t T = (size_t)gridDim.x * blockDim.x;
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll 1
  for (size_t i = t; i < groups; i += T) {
    float R[V], G[V], B[V], Y[V], Uo[V], Vo[V];
    mem::load_vec<float, V, true>(r, i * V, R);
    mem::load_vec<float, V, true>(g, i * V, G);
    mem::load_vec<float, V, true>(b, i * V, B);
#pragma unroll
    for (int l = 0; l < V; ++l) yuv<F>::px(R[l], G[l], B[l], Y[l], Uo[l], Vo[l]);
    mem::store_vec<float, V>(y, i * V, Y);
    mem::store_vec<float, V>(u, i * V, Uo);
    mem::store_vec<float, V>(v, i * V, Vo);
  }
  const size_t k = groups * V + t;
  if (k < n) yuv<F>::px(r[k], g[k], b[k], y[k], u[k], v[k]);
}

template <bool F>
__global__ void __launch_bounds__(256) k_rgb2yuv_scalar(const float* r, const float* g, const float* b, float* y,
                                                        float* u, float* v, size_t n)
{
  nt2cuda::mem::pdl_begin();
  const size_t T = (size_t)gridDim.x * blockDim.x;
#pragma unroll 1
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += T)
    yuv<F>::px(r[k], g[k], b[k], y[k], u[k], v[k]);
}

inline bool overlap(const void* a, const void* b, size_t bytes)
{
  const uintptr_t x = (uintptr_t)a, z = (uintptr_t)b;
  return x < z + bytes && z < x + bytes;
}

template <bool F> nt2cuda_status rgb2yuv_impl(const float* r, const float* g, const float* b, float* y,
                                              float* u, float* v, size_t n, cudaStream_t s)
{
  if (!n) return NT2CUDA_OK;
  // one fused pass reads every input before writing: outputs may overlap nothing
  const size_t bytes = n * sizeof(float);
  const void* outs[3] = {y, u, v};
  const void* all[6] = {r, g, b, y, u, v};
  for (int o = 0; o < 3; ++o)
    for (int k = 0; k < 6; ++k)
      if (k != o + 3 && overlap(outs[o], all[k], bytes)) return NT2CUDA_ERR_ALIAS;
  void* args[] = {(void*)&r, (void*)&g, (void*)&b, (void*)&y, (void*)&u, (void*)&v, (void*)&n};
  const uintptr_t bits = (uintptr_t)r | (uintptr_t)g | (uintptr_t)b | (uintptr_t)y | (uintptr_t)u | (uintptr_t)v;
  if (bits & 15u)       // a misaligned view: one element per thread
    return launch_status(launch_persistent(k_rgb2yuv_scalar<F>, n, 256, 2, s, args));
  return launch_status(launch_persistent(k_rgb2yuv<F>, n / 4 + 1, 256, 2, s, args));
}

// The demo statement.  Aligned tables (R the same table as an input, or
// disjoint from all of them) take one pass of k_bs_demo, the demo's local
// tables da, d1, d2 in registers.  Otherwise it is lowered through the
// generic expression engine, which rejects partial overlaps: d1 appears twice
// in R's tree (in d2 and in fastnormcdf(d1)), and a tree evaluates each
// occurrence; so d1 is its own statement into stream scratch, as the demo
// itself materialises it, and R's statement reads it.
template <bool F> nt2cuda_status bs_demo_impl(const float* S, const float* X, const float* T, const float* r,
                                              const float* v, float* R, size_t n, nt2cuda_stream s)
{
  if (n == 0) return NT2CUDA_OK;
  {
    const float* in[5] = {S, X, T, r, v};
    bool ok = ((uintptr_t)S | (uintptr_t)X | (uintptr_t)T | (uintptr_t)r | (uintptr_t)v | (uintptr_t)R) % 16u == 0 &&
              n <= ((size_t)1 << 60);
    for (int k = 0; k < 5 && ok; ++k) ok = in[k] == R || !overlap(in[k], R, n * sizeof(float));
    if (ok) {
      void* args[] = {(void*)&S, (void*)&X, (void*)&T, (void*)&r, (void*)&v, (void*)&R, (void*)&n};
      tuning::params def;
      def.unroll = 1;
      def.waves = 4;
      const tuning::params tp = tuning::lookup("bs_demo_f32", n, def);
      if (tp.unroll == 2)
        return launch_status(launch_persistent(k_bs_demo<F, 2>, n / 4 + 1, 256, tp.waves, as_stream(s), args));
      return launch_status(launch_persistent(k_bs_demo<F, 1>, n / 4 + 1, 256, tp.waves, as_stream(s), args));
    }
  }
  auto Sa = tm(S); auto Xa = tm(X); auto Ta = tm(T); auto ra = tm(r); auto va = tm(v);
  auto da = nd<tag::sqrt_>(Ta);
  // log(Sa/Xa) + (fma(sqr(va),0.5,ra)*Ta)/(va*da)
  auto d1 = nd<tag::plus_>(nd<tag::log_>(nd<tag::divides_>(Sa, Xa)),
                           nd<tag::divides_>(nd<tag::multiplies_>(nd<tag::fma_>(nd<tag::sqr_>(va), sc(0.5f), ra), Ta),
                                             nd<tag::multiplies_>(va, da)));
  void* scratch = nullptr;
  const cudaError_t e = nt2cuda::stream_scratch(as_stream(s), n * sizeof(float), &scratch, 1);
  if (e != cudaSuccess) return from_cuda(e);
  float* D1 = static_cast<float*>(scratch);
  const nt2cuda_status st = run<F>(make_prog(asg(D1, d1)), n, s, "bs_demo_d1_f32");
  if (st != NT2CUDA_OK) return st;
  auto d1t = tm(static_cast<const float*>(D1));
  auto d2 = nd<tag::fnms_>(va, da, d1t);
  auto R0 = nd<tag::fnms_>(nd<tag::multiplies_>(Xa, nd<tag::exp_>(nd<tag::multiplies_>(nd<tag::unary_minus_>(ra), Ta))),
                           nd<tag::fastnormcdf_>(d2),
                           nd<tag::multiplies_>(Sa, nd<tag::fastnormcdf_>(d1t)));
  return run<F>(make_prog(asg(R, R0)), n, s, "bs_demo_f32");
}

template <class T> bool aligned16(const T* p) { return ((uintptr_t)p & 15u) == 0; }

template <class T, int CDF, int P>
nt2cuda_status bs_launch(const T* S, const T* K, const T* Tm, T r, T v, T* call, T* put, size_t n,
                         cudaStream_t s, int unroll, int waves)
{
  if (n == 0) return NT2CUDA_OK;
  size_t nn = n;
  void* args[] = {(void*)&S, (void*)&K, (void*)&Tm, (void*)&r, (void*)&v, (void*)&call, (void*)&put, (void*)&nn};
  if (!(aligned16(S) && aligned16(K) && aligned16(Tm) && aligned16(call) && aligned16(put)))
    return launch_status(launch_persistent(k_blackscholes_scalar<T, CDF, P>, n, 256, waves, s, args));
  constexpr int V = 16 / (int)sizeof(T);
  size_t groups = n / V;
  switch (unroll) {
    case 1: return launch_status(launch_persistent(k_blackscholes<T, CDF, P, 1>, groups, 256, waves, s, args));
    case 4: return launch_status(launch_persistent(k_blackscholes<T, CDF, P, 4>, groups, 256, waves, s, args));
    default: return launch_status(launch_persistent(k_blackscholes<T, CDF, P, 2>, groups, 256, waves, s, args));
  }
}

template <class T, int CDF>
nt2cuda_status bs_prec(const T* S, const T* K, const T* Tm, T r, T v, T* call, T* put, size_t n, int prec,
                       cudaStream_t s, int unroll, int waves)
{
  switch (prec) {
    case PREC_EXACT: return bs_launch<T, CDF, PREC_EXACT>(S, K, Tm, r, v, call, put, n, s, unroll, waves);
    case PREC_FUSED: return bs_launch<T, CDF, PREC_FUSED>(S, K, Tm, r, v, call, put, n, s, unroll, waves);
    case PREC_FAST:
      if constexpr (sizeof(T) == 4) return bs_launch<T, CDF, PREC_FAST>(S, K, Tm, r, v, call, put, n, s, unroll, waves);
      else return NT2CUDA_ERR_ARG;
    default: return NT2CUDA_ERR_ARG;
  }
}

template <class T>
nt2cuda_status bs_dispatch(const T* S, const T* K, const T* Tm, T r, T v, T* call, T* put, size_t n,
                           int cdf, int prec, cudaStream_t s, int unroll, int waves)
{
  if (n && (!S || !K || !Tm || !call || !put)) return NT2CUDA_ERR_ARG;
  if (cdf != CDF_NORMCDF && cdf != CDF_FASTNORMCDF) return NT2CUDA_ERR_ARG;
  if constexpr (sizeof(T) == 8) {
    if (cdf != CDF_NORMCDF) return NT2CUDA_ERR_ARG;
    return bs_prec<T, CDF_NORMCDF>(S, K, Tm, r, v, call, put, n, prec, s, unroll, waves);
  } else {
    if (cdf == CDF_FASTNORMCDF) return bs_prec<T, CDF_FASTNORMCDF>(S, K, Tm, r, v, call, put, n, prec, s, unroll, waves);
    return bs_prec<T, CDF_NORMCDF>(S, K, Tm, r, v, call, put, n, prec, s, unroll, waves);
  }
}

template <int CDF, int P> void warm_bs()
{
  (void)resident_blocks(k_blackscholes<float, CDF, P, 1>, 256);
  (void)resident_blocks(k_blackscholes<float, CDF, P, 2>, 256);
  (void)resident_blocks(k_blackscholes<float, CDF, P, 4>, 256);
  (void)resident_blocks(k_blackscholes_scalar<float, CDF, P>, 256);
}

const char* bs_key(size_t bytes, int prec = 0)
{
  if (bytes != 4) return prec == PREC_FUSED ? "bs_f64_fused" : "bs_f64";
  return prec == PREC_FAST ? "bs_f32_fast" : (prec == PREC_FUSED ? "bs_f32_fused" : "bs_f32");
}

// ---------------------------------------------- host-buffer pipeline state
struct host_pipeline {
  std::mutex m;
  static constexpr int NS = 3;
  cudaStream_t st[NS] = {nullptr, nullptr, nullptr};
  float* buf[NS][5] = {};
  size_t chunk = 0;
  int dev = -1;
};
host_pipeline& hp() { static host_pipeline p; return p; }

}  // namespace

void nt2cuda::detail_capi::warm_blackscholes_f32(int cdf, int prec)
{
  if (cdf == CDF_FASTNORMCDF)
    prec == PREC_FAST ? warm_bs<CDF_FASTNORMCDF, PREC_FAST>()
    : prec == PREC_FUSED ? warm_bs<CDF_FASTNORMCDF, PREC_FUSED>() : warm_bs<CDF_FASTNORMCDF, PREC_EXACT>();
  else
    prec == PREC_FAST ? warm_bs<CDF_NORMCDF, PREC_FAST>()
    : prec == PREC_FUSED ? warm_bs<CDF_NORMCDF, PREC_FUSED>() : warm_bs<CDF_NORMCDF, PREC_EXACT>();
}

extern "C" {

nt2cuda_status nt2cuda_map_f32(int op, const float* x, float* y, size_t n, int flags, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!x || !y)) return NT2CUDA_ERR_ARG;
  if (flags & ~(NT2CUDA_MAP_FUSED | NT2CUDA_MAP_SIMD128)) return NT2CUDA_ERR_ARG;
  const bool fused = (flags & NT2CUDA_MAP_FUSED) != 0;
  if (op >= NT2CUDA_OP_SIN && op <= NT2CUDA_OP_TANH)
    return map_trig(op, x, y, n, fused, (flags & NT2CUDA_MAP_SIMD128) != 0, s);
  if ((op >= NT2CUDA_OP_CBRT && op <= NT2CUDA_OP_REALLOG) || (op >= NT2CUDA_OP_ATANH && op <= NT2CUDA_OP_SINHC))
    return map_expfam(op, x, y, n, fused, s);
  if ((op >= NT2CUDA_OP_CSC && op <= NT2CUDA_OP_SINCPI) || op == NT2CUDA_OP_PROPER_TANPI)
    return map_trigx(op, x, y, n, fused, (flags & NT2CUDA_MAP_SIMD128) != 0, s);
  return fused ? map_impl<true>(op, x, y, n, s) : map_impl<false>(op, x, y, n, s);
}

nt2cuda_status nt2cuda_map_f64(int op, const double* x, double* y, size_t n, int flags, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!x || !y)) return NT2CUDA_ERR_ARG;
  if (flags & ~(NT2CUDA_MAP_FUSED | NT2CUDA_MAP_SIMD128)) return NT2CUDA_ERR_ARG;
  const bool fused = (flags & NT2CUDA_MAP_FUSED) != 0;
  if (op >= NT2CUDA_OP_SIN && op <= NT2CUDA_OP_TANH)
    return map_trig(op, x, y, n, fused, (flags & NT2CUDA_MAP_SIMD128) != 0, s);
  if ((op >= NT2CUDA_OP_CBRT && op <= NT2CUDA_OP_REALLOG) || (op >= NT2CUDA_OP_ATANH && op <= NT2CUDA_OP_SINHC))
    return map_expfam(op, x, y, n, fused, s);
  if ((op >= NT2CUDA_OP_CSC && op <= NT2CUDA_OP_SINCPI) || op == NT2CUDA_OP_PROPER_TANPI)
    return map_trigx(op, x, y, n, fused, (flags & NT2CUDA_MAP_SIMD128) != 0, s);
  return fused ? map_impl<true>(op, x, y, n, s) : map_impl<false>(op, x, y, n, s);
}

nt2cuda_status nt2cuda_saxpy_f32(float a, const float* x, float* y, size_t n, int fused, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!x || !y)) return NT2CUDA_ERR_ARG;
  return fused ? saxpy_impl<true>(a, x, y, n, s) : saxpy_impl<false>(a, x, y, n, s);
}

nt2cuda_status nt2cuda_saxpy_f64(double a, const double* x, double* y, size_t n, int fused, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!x || !y)) return NT2CUDA_ERR_ARG;
  return fused ? saxpy_impl<true>(a, x, y, n, s) : saxpy_impl<false>(a, x, y, n, s);
}

nt2cuda_status nt2cuda_rgb2grey_f32(const float* r, const float* g, const float* b, float* gr, size_t n,
                                    int fused, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!r || !g || !b || !gr)) return NT2CUDA_ERR_ARG;
  return fused ? rgb2grey_impl<true>(r, g, b, gr, n, s) : rgb2grey_impl<false>(r, g, b, gr, n, s);
}

nt2cuda_status nt2cuda_rgb2grey_u8(const uint8_t* r, const uint8_t* g, const uint8_t* b, uint8_t* gr, size_t n,
                                   int fused, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!r || !g || !b || !gr)) return NT2CUDA_ERR_ARG;
  return fused ? rgb2grey_u8_impl<true>(r, g, b, gr, n, s) : rgb2grey_u8_impl<false>(r, g, b, gr, n, s);
}

nt2cuda_status nt2cuda_rgb2yuv_f32(const float* r, const float* g, const float* b, float* y, float* u, float* v,
                                   size_t n, int fused, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!r || !g || !b || !y || !u || !v)) return NT2CUDA_ERR_ARG;
  return fused ? rgb2yuv_impl<true>(r, g, b, y, u, v, n, as_stream(s))
               : rgb2yuv_impl<false>(r, g, b, y, u, v, n, as_stream(s));
}

nt2cuda_status nt2cuda_blackscholes_demo_f32(const float* S, const float* X, const float* T, const float* r,
                                             const float* v, float* R, size_t n, int fused, nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  if (n && (!S || !X || !T || !r || !v || !R)) return NT2CUDA_ERR_ARG;
  return fused ? bs_demo_impl<true>(S, X, T, r, v, R, n, s) : bs_demo_impl<false>(S, X, T, r, v, R, n, s);
}

nt2cuda_status nt2cuda_blackscholes_f32(const float* S, const float* K, const float* T, float r, float sigma,
                                        float* call, float* put, size_t n, int cdf_kind, int fused,
                                        nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  tuning::params p = tuning::lookup(bs_key(4, fused), n);
  return bs_dispatch<float>(S, K, T, r, sigma, call, put, n, cdf_kind, fused, as_stream(s), p.unroll, p.waves);
}

nt2cuda_status nt2cuda_blackscholes_f64(const double* S, const double* K, const double* T, double r,
                                        double sigma, double* call, double* put, size_t n, int fused,
                                        nt2cuda_stream s)
{
  NT2CUDA_NVTX_RANGE;
  tuning::params p = tuning::lookup(bs_key(8, fused), n);
  return bs_dispatch<double>(S, K, T, r, sigma, call, put, n, CDF_NORMCDF, fused, as_stream(s), p.unroll,
                             p.waves);
}

}  // extern "C"

namespace {

// Device-side address of a pinned (page-locked, mapped) host buffer, or null.
template <class T> T* mapped_ptr(T* p)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr || a.hostPointer == nullptr) return nullptr;
  return (T*)((char*)a.devicePointer + ((const char*)p - (const char*)a.hostPointer));
}

// Which host path to take: 0 = automatic (mapped when every table is pinned),
// 1 = always staged copies, 2 = mapped whenever possible.  Read once from
// NT2CUDA_HOST_PATH ("auto", "staged", "mapped").
int host_path_policy()
{
  static int policy = [] {
    const char* e = getenv("NT2CUDA_HOST_PATH");
    if (!e) return 0;
    if (!strcmp(e, "staged")) return 1;
    if (!strcmp(e, "mapped")) return 2;
    return 0;
  }();
  return policy;
}

}  // namespace

extern "C" {

nt2cuda_status nt2cuda_blackscholes_f32_host(const float* S, const float* K, const float* T, float r,
                                             float sigma, float* call, float* put, size_t n, int cdf_kind,
                                             int fused)
{
  NT2CUDA_NVTX_RANGE;
  if (n == 0) return NT2CUDA_OK;
  if (!S || !K || !T || !call || !put) return NT2CUDA_ERR_ARG;
  host_pipeline& P = hp();
  std::lock_guard<std::mutex> g(P.m);
  int dev = 0;
  cudaGetDevice(&dev);
  const int policy = host_path_policy();
  // Mapped path: pinned host tables are read and written by the kernel in place over
  // NVLink-C2C (no staging copies, no HBM round trip).
  const float *mS = nullptr, *mK = nullptr, *mT = nullptr;
  float *mc = nullptr, *mp = nullptr;
  if (policy != 1) {
    mS = mapped_ptr(S); mK = mapped_ptr(K); mT = mapped_ptr(T); mc = mapped_ptr(call); mp = mapped_ptr(put);
  }
  if (mS && mK && mT && mc && mp) {
    if (!P.st[0]) {
      cudaError_t e = cudaStreamCreateWithFlags(&P.st[0], cudaStreamNonBlocking);
      if (e != cudaSuccess) return from_cuda(e);
    }
    tuning::params tp = tuning::lookup(fused == PREC_FAST ? "bs_f32_fast_mapped" : "bs_f32_mapped", n);
    nt2cuda_status rs = bs_dispatch<float>(mS, mK, mT, r, sigma, mc, mp, n, cdf_kind, fused, P.st[0], tp.unroll,
                                           tp.waves);
    if (rs != NT2CUDA_OK) return rs;
    return from_cuda(cudaStreamSynchronize(P.st[0]));
  }
  const size_t chunk = (size_t)1 << 21;   // options per pipeline stage (8 MiB per table)
  if (P.dev != dev || P.chunk < chunk) {
    for (int i = 0; i < host_pipeline::NS; ++i) {
      for (int j = 0; j < 5; ++j) { if (P.buf[i][j]) cudaFree(P.buf[i][j]); P.buf[i][j] = nullptr; }
      if (P.st[i]) cudaStreamDestroy(P.st[i]);
      P.st[i] = nullptr;
    }
    P.chunk = 0;
    P.dev = -1;
    for (int i = 0; i < host_pipeline::NS; ++i) {
      cudaError_t e = cudaStreamCreateWithFlags(&P.st[i], cudaStreamNonBlocking);
      if (e != cudaSuccess) return from_cuda(e);
      for (int j = 0; j < 5; ++j) {
        e = cudaMalloc(&P.buf[i][j], chunk * sizeof(float));
        if (e != cudaSuccess) return from_cuda(e);
      }
    }
    P.chunk = chunk;
    P.dev = dev;
  }
  tuning::params tp = tuning::lookup(bs_key(4, fused), chunk);
  size_t nchunks = (n + chunk - 1) / chunk;
  for (size_t c = 0; c < nchunks; ++c) {
    int i = (int)(c % host_pipeline::NS);
    cudaStream_t st = P.st[i];
    size_t off = c * chunk, cnt = (n - off) < chunk ? (n - off) : chunk;
    size_t b = cnt * sizeof(float);
    float** d = P.buf[i];
    cudaMemcpyAsync(d[0], S + off, b, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d[1], K + off, b, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d[2], T + off, b, cudaMemcpyHostToDevice, st);
    nt2cuda_status rs = bs_dispatch<float>(d[0], d[1], d[2], r, sigma, d[3], d[4], cnt, cdf_kind, fused, st,
                                           tp.unroll, tp.waves);
    if (rs != NT2CUDA_OK) { for (int k = 0; k < host_pipeline::NS; ++k) cudaStreamSynchronize(P.st[k]); return rs; }
    cudaMemcpyAsync(call + off, d[3], b, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(put + off, d[4], b, cudaMemcpyDeviceToHost, st);
  }
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < host_pipeline::NS; ++i) {
    cudaError_t e = cudaStreamSynchronize(P.st[i]);
    if (e != cudaSuccess) err = e;
  }
  return from_cuda(err);
}

// ------------------------------------------------------------ autotuner
nt2cuda_status nt2cuda_autotune(const char* kernel, size_t n, int* best_unroll, int* best_waves, float* best_ms)
{
  if (!kernel || n == 0) return NT2CUDA_ERR_ARG;
  std::string k(kernel);
  const bool f64 = (k == "bs_f64" || k == "bs_f64_fused" || k == "saxpy_f64");
  const bool grey8 = (k == "rgb2grey_u8");
  const size_t es = f64 ? 8 : (grey8 ? 1 : 4);
  int prec = PREC_EXACT;
  if (k == "bs_f32_fused" || k == "bs_f64_fused") prec = PREC_FUSED;
  if (k == "bs_f32_fast" || k == "bs_f32_fast_mapped") prec = PREC_FAST;
  // *_mapped keys tune the kernel on pinned host tables (the zero-copy host path)
  const bool mapped = (k == "bs_f32_mapped" || k == "bs_f32_fast_mapped");
  const bool bs32 = (k == "bs_f32" || k == "bs_f32_fused" || k == "bs_f32_fast" || mapped);
  const bool bs64 = (k == "bs_f64" || k == "bs_f64_fused");
  if (!(bs32 || bs64 || grey8 || k == "saxpy_f32" || k == "saxpy_f64")) return NT2CUDA_ERR_ARG;
  void* buf[5] = {};
  for (int j = 0; j < 5; ++j) {
    cudaError_t e = mapped ? cudaMallocHost(&buf[j], n * es) : cudaMalloc(&buf[j], n * es);
    if (e != cudaSuccess) {
      for (int q = 0; q < j; ++q) { if (mapped) cudaFreeHost(buf[q]); else cudaFree(buf[q]); }
      return from_cuda(e);
    }
  }
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (grey8) {
    for (int j = 0; j < 3; ++j) cudaMemsetAsync(buf[j], 0x5a + 40 * j, n, s);
  } else if (f64) {
    nt2cuda_fill_uniform_f64((double*)buf[0], n, 5.0, 30.0, 1, s);
    nt2cuda_fill_uniform_f64((double*)buf[1], n, 1.0, 100.0, 2, s);
    nt2cuda_fill_uniform_f64((double*)buf[2], n, 0.25, 10.0, 3, s);
  } else {
    nt2cuda_fill_uniform_f32((float*)buf[0], n, 5.0f, 30.0f, 1, s);
    nt2cuda_fill_uniform_f32((float*)buf[1], n, 1.0f, 100.0f, 2, s);
    nt2cuda_fill_uniform_f32((float*)buf[2], n, 0.25f, 10.0f, 3, s);
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int unrolls[3] = {1, 2, 4};
  const int wavesv[4] = {1, 2, 4, 8};
  float best = 1e30f;
  tuning::params bp;
  nt2cuda_status st = NT2CUDA_OK;
  for (int ui = 0; ui < 3 && st == NT2CUDA_OK; ++ui)
    for (int wi = 0; wi < 4 && st == NT2CUDA_OK; ++wi) {
      auto once = [&]() -> nt2cuda_status {
        if (bs32)
          return bs_dispatch<float>((float*)buf[0], (float*)buf[1], (float*)buf[2], 0.02f, 0.30f, (float*)buf[3],
                                    (float*)buf[4], n, CDF_NORMCDF, prec, s, unrolls[ui], wavesv[wi]);
        if (bs64)
          return bs_dispatch<double>((double*)buf[0], (double*)buf[1], (double*)buf[2], 0.02, 0.30,
                                     (double*)buf[3], (double*)buf[4], n, CDF_NORMCDF, prec, s, unrolls[ui],
                                     wavesv[wi]);
        tuning::set(k.c_str(), n, tuning::params{unrolls[ui], wavesv[wi]});
        if (grey8)
          return nt2cuda_rgb2grey_u8((const uint8_t*)buf[0], (const uint8_t*)buf[1], (const uint8_t*)buf[2],
                                     (uint8_t*)buf[3], n, 0, s);
        if (k == "saxpy_f32") return nt2cuda_saxpy_f32(2.5f, (float*)buf[0], (float*)buf[1], n, 0, s);
        return nt2cuda_saxpy_f64(2.5, (double*)buf[0], (double*)buf[1], n, 0, s);
      };
      for (int w = 0; w < 2 && st == NT2CUDA_OK; ++w) st = once();
      cudaEventRecord(e0, s);
      const int reps = 5;
      for (int rr = 0; rr < reps && st == NT2CUDA_OK; ++rr) st = once();
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      if (ms < best) { best = ms; bp = tuning::params{unrolls[ui], wavesv[wi]}; }
    }
  if (st == NT2CUDA_OK) tuning::set(k.c_str(), n, bp);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  for (int j = 0; j < 5; ++j) { if (mapped) cudaFreeHost(buf[j]); else cudaFree(buf[j]); }
  if (st != NT2CUDA_OK) return st;
  if (best_unroll) *best_unroll = bp.unroll;
  if (best_waves) *best_waves = bp.waves;
  if (best_ms) *best_ms = best;
  return NT2CUDA_OK;
}

}  // extern "C"
