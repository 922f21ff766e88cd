// nt2cuda/blackscholes.cuh -- the Black-Scholes call/put statement lowered
// by hand into one kernel.
//
// NT2 user code:
//   da  = sqrt(T);  vda = v*da;
//   d1  = (log(S/K) + fma(sqr(v),0.5,r)*T) / vda;   d2 = d1 - vda;
//   e   = K*exp(-r*T);
//   tie(call, put) = tie(fnms(e, normcdf(d2), S*normcdf(d1)),
//                        fnms(S, normcdf(-d1), e*normcdf(-d2)));
// (modules/core/container/table/include/nt2/core/functions/expr/tie.hpp:40-74 for tie,
//  demo/blackscholes/nt2_merged/blackandscholes_nt2_merged.cpp:57-64 for the merged form).
// The generic lowering in expr.cuh would evaluate four erfc; here normcdf(x)
// and normcdf(-x) share one erfc core (math::normcdf_pair), which is
// bit-identical because NT2's erfc only uses the sign and |argument|.  The
// scalar subexpression fma(sqr(v),0.5,r) is formed once per thread; NT2
// forms it per element from the same splatted scalars, with the same result.
// The proto optimizer's a + b*c -> fma(b,c,a) rewrite
// (modules/boost/simd/base/include/boost/simd/operator/functions/optimize/plus.hpp:20-45)
// applies to log(S/K) + c*T, which is why that sum is a madd.
//
// Exact FP32 normcdf options are priced two at a time on the packed FP32
// instructions (nt2cuda/bs_x2.cuh), bit-identical to bs_lane.
#pragma once
#include <cuda_runtime.h>
#include "bs_x2.cuh"
#include "math.cuh"
#include "memory.cuh"

namespace nt2cuda {

enum { CDF_NORMCDF = 0, CDF_FASTNORMCDF = 1 };
// Precision modes: 0 = NT2's arithmetic unfused (bit-exact), 1 = each NT2
// fma/fnms/Horner step as one hardware FMA, 2 = fast (FMA, and the
// special-function unit for exp, log, rsqrt and reciprocals; NT2's erfc and
// fastnormcdf polynomials; float only).
enum { PREC_EXACT = 0, PREC_FUSED = 1, PREC_FAST = 2 };

template <class T, int CDF, int P>
__device__ __forceinline__ void bs_lane(T S, T K, T Tm, T r, T v, T c, T& call, T& put)
{
  using namespace math;
  constexpr bool F = P != PREC_EXACT;
  if constexpr (P == PREC_FAST && sizeof(T) == 4) {
    // sqrt(T) = T * rsqrt(T) and the divisions by reciprocal on the special-function unit
    const float rs = rsqrtf(Tm);
    const float vda = __fmul_rn(v, __fmul_rn(Tm, rs));
    const float d1 = __fdividef(__fmaf_rn(c, Tm, fast::log(__fdividef(S, K))), vda);
    const float d2 = __fsub_rn(d1, vda);
    const float e = __fmul_rn(K, fast::exp_small(__fmul_rn(-r, Tm)));
    float n1, m1, n2, m2;
    if constexpr (CDF == CDF_FASTNORMCDF) {
      fast::fastnormcdf_pair(d1, n1, m1);
      fast::fastnormcdf_pair(d2, n2, m2);
    } else {
      fast::normcdf_pair(d1, n1, m1);
      fast::normcdf_pair(d2, n2, m2);
    }
    call = __fmaf_rn(-e, n2, __fmul_rn(S, n1));
    put = __fmaf_rn(-S, m1, __fmul_rn(e, m2));
    return;
  }
  T da = sqrt_(Tm);
  T vda = mul(v, da);
  T d1 = div(madd<F>(c, Tm, log<F>(div(S, K))), vda);
  T d2 = sub(d1, vda);
  T e = mul(K, exp<F>(mul(-r, Tm)));
  T n1, m1, n2, m2;
  if constexpr (CDF == CDF_FASTNORMCDF) {
    fastnormcdf_pair<F>(d1, n1, m1);
    fastnormcdf_pair<F>(d2, n2, m2);
  } else {
    normcdf_pair<F>(d1, n1, m1);
    normcdf_pair<F>(d2, n2, m2);
  }
  call = nmsub<F>(e, n2, mul(S, n1));
  put = nmsub<F>(S, m1, mul(e, m2));
}

// Statements priced two options at a time (bs_x2.cuh): FP32, normcdf or
// fastnormcdf, exact or fused (each NT2 fma/fnms one hardware FMA, as bs_lane's).
template <class T, int CDF, int P>
constexpr bool kPacked = sizeof(T) == 4 && (P == PREC_EXACT || P == PREC_FUSED);
// ... and the fast mode's statement (x2::fast), bit-identical to bs_lane's fast branch.
template <class T, int CDF, int P>
constexpr bool kPackedFast = sizeof(T) == 4 && CDF == CDF_NORMCDF && P == PREC_FAST;

// V options per thread per group (16 bytes of each input), U groups in
// flight per grid-stride trip.
// The packed form is held to the registers of 5, 4 and 2 resident blocks per
// SM at U = 1, 2, 4, so that its independent option pairs come with enough
// warps to hide the FP32 pipes' latency (0: the compiler's own choice).
template <class T, int CDF, int P, int U>
constexpr int kMinBlocks = !kPacked<T, CDF, P> ? 0 : (U == 1 ? 5 : (U == 2 ? 4 : 2));

template <class T, int CDF, int P, int U>
__global__ void __launch_bounds__(256, (kMinBlocks<T, CDF, P, U>))
    k_blackscholes(const T* __restrict__ S, const T* __restrict__ K,
                                                      const T* __restrict__ Tm, T r, T v,
                                                      T* __restrict__ call, T* __restrict__ put, size_t n)
{
  nt2cuda::mem::pdl_begin();
  constexpr int V = 16 / (int)sizeof(T);
  const T c = math::madd<(P != PREC_EXACT)>(math::mul(v, v), T(0.5), r);
  const size_t ngroups = n / V;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t g = tid;
#pragma unroll 1
  for (; g + (size_t)(U - 1) * stride < ngroups; g += (size_t)U * stride) {
    T s[U][V], k[U][V], t[U][V];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      size_t i = (g + (size_t)u * stride) * V;
      mem::load_vec<T, V, true>(S, i, s[u]);
      mem::load_vec<T, V, true>(K, i, k[u]);
      mem::load_vec<T, V, true>(Tm, i, t[u]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      T oc[V], op[V];
      if constexpr (kPacked<T, CDF, P> || kPackedFast<T, CDF, P>) {
#pragma unroll
        for (int l = 0; l < V; l += 2) {
          float2 pc, pp;
          const float2 ps = make_float2(s[u][l], s[u][l + 1]), pk = make_float2(k[u][l], k[u][l + 1]),
                       pt = make_float2(t[u][l], t[u][l + 1]);
          if constexpr (kPackedFast<T, CDF, P>) x2::fast::blackscholes(ps, pk, pt, r, v, c, pc, pp);
          else if constexpr (CDF == CDF_FASTNORMCDF)
            x2::blackscholes_fastnormcdf<P == PREC_FUSED>(ps, pk, pt, r, v, c, pc, pp);
          else x2::blackscholes<P == PREC_FUSED>(ps, pk, pt, r, v, c, pc, pp);
          oc[l] = pc.x; oc[l + 1] = pc.y;
          op[l] = pp.x; op[l + 1] = pp.y;
        }
      } else {
#pragma unroll
        for (int l = 0; l < V; ++l) bs_lane<T, CDF, P>(s[u][l], k[u][l], t[u][l], r, v, c, oc[l], op[l]);
      }
      size_t i = (g + (size_t)u * stride) * V;
      mem::store_vec<T, V>(call, i, oc);
      mem::store_vec<T, V>(put, i, op);
    }
  }
#pragma unroll 1
  for (; g < ngroups; g += stride) {
    T s[V], k[V], t[V], oc[V], op[V];
    size_t i = g * V;
    mem::load_vec<T, V, true>(S, i, s);
    mem::load_vec<T, V, true>(K, i, k);
    mem::load_vec<T, V, true>(Tm, i, t);
    if constexpr (kPacked<T, CDF, P> || kPackedFast<T, CDF, P>) {
#pragma unroll
      for (int l = 0; l < V; l += 2) {
        float2 pc, pp;
        const float2 ps = make_float2(s[l], s[l + 1]), pk = make_float2(k[l], k[l + 1]), pt = make_float2(t[l], t[l + 1]);
        if constexpr (kPackedFast<T, CDF, P>) x2::fast::blackscholes(ps, pk, pt, r, v, c, pc, pp);
        else if constexpr (CDF == CDF_FASTNORMCDF)
          x2::blackscholes_fastnormcdf<P == PREC_FUSED>(ps, pk, pt, r, v, c, pc, pp);
        else x2::blackscholes<P == PREC_FUSED>(ps, pk, pt, r, v, c, pc, pp);
        oc[l] = pc.x; oc[l + 1] = pc.y;
        op[l] = pp.x; op[l + 1] = pp.y;
      }
    } else {
#pragma unroll
      for (int l = 0; l < V; ++l) bs_lane<T, CDF, P>(s[l], k[l], t[l], r, v, c, oc[l], op[l]);
    }
    mem::store_vec<T, V>(call, i, oc);
    mem::store_vec<T, V>(put, i, op);
  }
  const size_t tail0 = ngroups * V;
  if (tid < n - tail0) {
    size_t i = tail0 + tid;
    bs_lane<T, CDF, P>(S[i], K[i], Tm[i], r, v, c, call[i], put[i]);
  }
}

// The demo form of the statement (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59),
// five FP32 tables in and R out:
//   da = sqrt(Ta);  d1 = log(Sa/Xa) + (fma(sqr(va),0.5,ra)*Ta)/(va*da);
//   d2 = fnms(va,da,d1);
//   R  = fnms(Xa*exp(-ra*Ta), fastnormcdf(d2), Sa*fastnormcdf(d1));
// da, d1 and d2 are the demo's local tables, read only by the statements that
// follow them, so here they stay in registers: one pass reads the five inputs
// once and writes R.  Two options per packed instruction (bs_x2.cuh); every
// value is the one the statements give element by element (each product that
// feeds an add or subtract formed by x2::mul_r).
template <bool F>
__device__ __forceinline__ float2 bs_demo_pair(float2 S, float2 X, float2 T, float2 r, float2 v)
{
  const float2 da = make_float2(__fsqrt_rn(T.x), __fsqrt_rn(T.y));
  const float2 L = x2::log<F>(make_float2(__fdiv_rn(S.x, X.x), __fdiv_rn(S.y, X.y)));
  const float2 c = x2::madd<F>(x2::mul(v, v), x2::splat(0.5f), r);
  const float2 num = x2::mul(c, T), den = x2::mul(v, da);
  const float2 d1 = x2::add(L, make_float2(__fdiv_rn(num.x, den.x), __fdiv_rn(num.y, den.y)));
  const float2 d2 = x2::nmsub<F>(v, da, d1);
  const float2 e = x2::mul(X, x2::exp<F>(x2::mul_r(make_float2(-r.x, -r.y), T)));
  float2 n1, m1, n2, m2;
  x2::fastnormcdf_pair<F>(d2, n2, m2);
  x2::fastnormcdf_pair<F>(d1, n1, m1);
  return x2::nmsub<F>(e, n2, x2::mul_r(S, n1));
}

// Four options per thread per group (16 bytes of each table), U groups in
// flight per grid-stride trip; the last n % 4 options one per thread.
template <bool F, int U>
__global__ void __launch_bounds__(256, U == 1 ? 4 : 3)
    k_bs_demo(const float* __restrict__ S, const float* __restrict__ X, const float* __restrict__ T,
              const float* __restrict__ r, const float* __restrict__ v, float* __restrict__ R, size_t n)
{
  nt2cuda::mem::pdl_begin();
  constexpr int V = 4;
  const size_t ngroups = n / V;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t g = tid;
#pragma unroll 1
  for (; g + (size_t)(U - 1) * stride < ngroups; g += (size_t)U * stride) {
    float s[U][V], x[U][V], t[U][V], rr[U][V], vv[U][V];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const size_t i = (g + (size_t)u * stride) * V;
      mem::load_vec<float, V, true>(S, i, s[u]);
      mem::load_vec<float, V, true>(X, i, x[u]);
      mem::load_vec<float, V, true>(T, i, t[u]);
      mem::load_vec<float, V, true>(r, i, rr[u]);
      mem::load_vec<float, V, true>(v, i, vv[u]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float o[V];
#pragma unroll
      for (int l = 0; l < V; l += 2) {
        const float2 y = bs_demo_pair<F>(make_float2(s[u][l], s[u][l + 1]), make_float2(x[u][l], x[u][l + 1]),
                                         make_float2(t[u][l], t[u][l + 1]), make_float2(rr[u][l], rr[u][l + 1]),
                                         make_float2(vv[u][l], vv[u][l + 1]));
        o[l] = y.x;
        o[l + 1] = y.y;
      }
      mem::store_vec<float, V>(R, (g + (size_t)u * stride) * V, o);
    }
  }
#pragma unroll 1
  for (; g < ngroups; g += stride) {
    float s[V], x[V], t[V], rr[V], vv[V], o[V];
    const size_t i = g * V;
    mem::load_vec<float, V, true>(S, i, s);
    mem::load_vec<float, V, true>(X, i, x);
    mem::load_vec<float, V, true>(T, i, t);
    mem::load_vec<float, V, true>(r, i, rr);
    mem::load_vec<float, V, true>(v, i, vv);
#pragma unroll
    for (int l = 0; l < V; l += 2) {
      const float2 y = bs_demo_pair<F>(make_float2(s[l], s[l + 1]), make_float2(x[l], x[l + 1]),
                                       make_float2(t[l], t[l + 1]), make_float2(rr[l], rr[l + 1]),
                                       make_float2(vv[l], vv[l + 1]));
      o[l] = y.x;
      o[l + 1] = y.y;
    }
    mem::store_vec<float, V>(R, i, o);
  }
  const size_t tail0 = ngroups * V;
  if (tid < n - tail0) {   // one option, in both lanes of a pair (the lanes are independent)
    const size_t i = tail0 + tid;
    R[i] = bs_demo_pair<F>(make_float2(S[i], S[i]), make_float2(X[i], X[i]), make_float2(T[i], T[i]),
                           make_float2(r[i], r[i]), make_float2(v[i], v[i])).x;
  }
}

// Misaligned tables: one option per thread per trip.
template <class T, int CDF, int P>
__global__ void __launch_bounds__(256) k_blackscholes_scalar(const T* S, const T* K, const T* Tm, T r, T v,
                                                             T* call, T* put, size_t n)
{
  nt2cuda::mem::pdl_begin();
  const T c = math::madd<(P != PREC_EXACT)>(math::mul(v, v), T(0.5), r);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    bs_lane<T, CDF, P>(S[i], K[i], Tm[i], r, v, c, call[i], put[i]);
}

}  // namespace nt2cuda
