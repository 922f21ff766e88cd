// capi_selftest.cu -- exhaustive checks that the two-lane forms of NT2's
// float functors (nt2cuda/bs_x2.cuh) give the one-lane forms' bits
// (nt2cuda/math.cuh) for every float argument (for pow: every float as
// either argument, with drawn partners).
//
// Each check runs one kernel over all 2^32 float bit patterns (2^31 pairs),
// compares the packed result of both lanes with the scalar functor bit for
// bit (two NaNs count as equal: the results' contract covers NaN-ness, not
// payloads) and counts the differences.
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.cuh"
#include "nt2cuda/bs_x2.cuh"
#include "nt2cuda/launch.cuh"
#include "nt2cuda/math.cuh"
#include "nt2cuda/trig.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;

namespace {

__device__ __forceinline__ bool same(float a, float b)
{
  return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}

struct x2_report {
  unsigned long long mismatches;
  uint32_t first[8];
};

__device__ __forceinline__ void record(x2_report* rep, uint32_t u)
{
  const unsigned long long k = atomicAdd(&rep->mismatches, 1ull);
  if (k < 8) rep->first[k] = u;
}

// which: 0 exp, 1 log, 2 erfc of |a|, 3 normcdf(a) and normcdf(-a); 4..7 the
// same with each NT2 fma/fnms one hardware FMA (math::*<true>)
template <bool F> __device__ __forceinline__ void x2_check_pair(int which, uint32_t u0, x2_report* rep)
{
  const uint32_t u1 = u0 + 1;
  const float2 a = make_float2(__uint_as_float(u0), __uint_as_float(u1));
  if (which == 0) {
    const float2 r = x2::exp<F>(a);
    if (!same(r.x, math::exp<F>(a.x))) record(rep, u0);
    if (!same(r.y, math::exp<F>(a.y))) record(rep, u1);
  } else if (which == 1) {
    const float2 r = x2::log<F>(a);
    if (!same(r.x, math::log<F>(a.x))) record(rep, u0);
    if (!same(r.y, math::log<F>(a.y))) record(rep, u1);
  } else if (which == 2) {
    const float2 x = make_float2(fabsf(a.x), fabsf(a.y));
    const float2 r = x2::erfc_abs<F>(x);
    if (!same(r.x, math::erfc_abs<F>(x.x))) record(rep, u0);
    if (!same(r.y, math::erfc_abs<F>(x.y))) record(rep, u1);
  } else {
    float2 pos, neg;
    x2::normcdf_pair<F>(a, pos, neg);
    float p0, n0, p1, n1;
    math::normcdf_pair<F>(a.x, p0, n0);
    math::normcdf_pair<F>(a.y, p1, n1);
    if (!same(pos.x, p0) || !same(neg.x, n0)) record(rep, u0);
    if (!same(pos.y, p1) || !same(neg.y, n1)) record(rep, u1);
  }
}

// 8..11: the fast mode's exp_small, log, erfc(|a|) and normcdf pair (math::fast)
__device__ __forceinline__ void x2_check_fast(int which, uint32_t u0, x2_report* rep)
{
  const uint32_t u1 = u0 + 1;
  const float2 a = make_float2(__uint_as_float(u0), __uint_as_float(u1));
  if (which == 0) {
    const float2 r = x2::fast::exp_small(a);
    if (!same(r.x, math::fast::exp_small(a.x))) record(rep, u0);
    if (!same(r.y, math::fast::exp_small(a.y))) record(rep, u1);
  } else if (which == 1) {
    const float2 r = x2::fast::log(a);
    if (!same(r.x, math::fast::log(a.x))) record(rep, u0);
    if (!same(r.y, math::fast::log(a.y))) record(rep, u1);
  } else if (which == 2) {
    const float2 x = make_float2(fabsf(a.x), fabsf(a.y));
    const float2 r = x2::fast::erfc_abs_nr(x);
    if (!same(r.x, math::fast::erfc_abs_nr(x.x))) record(rep, u0);
    if (!same(r.y, math::fast::erfc_abs_nr(x.y))) record(rep, u1);
  } else {
    float2 pos, neg;
    x2::fast::normcdf_pair(a, pos, neg);
    float p0, n0, p1, n1;
    math::fast::normcdf_pair(a.x, p0, n0);
    math::fast::normcdf_pair(a.y, p1, n1);
    if (!same(pos.x, p0) || !same(neg.x, n0)) record(rep, u0);
    if (!same(pos.y, p1) || !same(neg.y, n1)) record(rep, u1);
  }
}

// 12, 13: fastnormcdf(a) and fastnormcdf(-a), NT2's arithmetic and fused
template <bool F> __device__ __forceinline__ void x2_check_fnc(uint32_t u0, x2_report* rep)
{
  const uint32_t u1 = u0 + 1;
  const float2 a = make_float2(__uint_as_float(u0), __uint_as_float(u1));
  float2 pos, neg;
  x2::fastnormcdf_pair<F>(a, pos, neg);
  float p0, n0, p1, n1;
  math::fastnormcdf_pair<F>(a.x, p0, n0);
  math::fastnormcdf_pair<F>(a.y, p1, n1);
  if (!same(pos.x, p0) || !same(neg.x, n0)) record(rep, u0);
  if (!same(pos.y, p1) || !same(neg.y, n1)) record(rep, u1);
}

// 14..21: the packed finish (trig::finish2) against finish, the bit pattern
// as the reduced argument, its low bits as the quadrant and bit 2 as the
// argument's sign: 14 sin, 15 cos, 16 and 17 the same fused; 18 tan, 19 cot,
// 20 and 21 the same fused
template <int K, bool F> __device__ __forceinline__ void x2_check_trig(uint32_t u0, x2_report* rep)
{
  const uint32_t u1 = u0 + 1;
  const float xr0 = __uint_as_float(u0), xr1 = __uint_as_float(u1);
  const int n0 = (int)(u0 & 3u), n1 = (int)(u1 & 3u);
  const float a0 = (u0 & 4u) ? -1.0f : 1.0f, a1 = (u1 & 4u) ? -1.0f : 1.0f;
  float y0, y1;
  trig::finish2<K, F>(a0, a1, xr0, xr1, n0, n1, y0, y1);
  if (!same(y0, trig::finish<K, F>(a0, xr0, n0))) record(rep, u0);
  if (!same(y1, trig::finish<K, F>(a1, xr1, n1))) record(rep, u1);
}

// 22..25: pow and pow_abs (22 pow, 23 pow fused, 24 pow_abs, 25 pow_abs
// fused) in two sweeps: the pair's bit patterns as a0 with an exponent drawn
// from a hash of them, then as a1 with a drawn base.  The draws mix random
// bit patterns, integers (odd and even), uniform values of both signs and
// special values, so that over the sweeps every float meets each kind of
// partner.
__device__ __forceinline__ uint32_t mix32(uint32_t h)
{
  h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
  return h;
}
__device__ __forceinline__ float draw(uint32_t u, bool base)
{
  const uint32_t h = mix32(u * 2u + (base ? 1u : 0u)), g = mix32(h);
  const float unit = (float)(g >> 8) * (1.0f / 16777216.0f);   // [0, 1)
  switch (h & 7u) {
    case 0: case 1: return __uint_as_float(g);                                 // any pattern
    case 2: return (float)((int)(g & 255u) - 128);                             // integer
    case 3: return base ? unit * 100.0f : (unit - 0.5f) * 20.0f;               // the bench's ranges
    case 4: return (unit - 0.5f) * 512.0f;                                     // wide
    case 5: return base ? 1.0f + (unit - 0.5f) * 1e-3f : (unit - 0.5f) * 1e-3f;   // near 1 / near 0
    case 6: {
      const float sp[8] = {0.0f, -0.0f, 1.0f, -1.0f, 0.5f, __int_as_float(0x7f800000),
                           __int_as_float(0xff800000), __int_as_float(0x7fc00000)};
      return sp[g & 7u];
    }
    default: return ldexpf(1.0f + unit, (int)(g & 63u) - 32) * ((g & 64u) ? -1.0f : 1.0f);
  }
}
template <bool ABS, bool F> __device__ __forceinline__ void x2_check_pow(uint32_t u0, x2_report* rep)
{
  const uint32_t u1 = u0 + 1;
  const float p0 = __uint_as_float(u0), p1 = __uint_as_float(u1);
#pragma unroll
  for (int sweep = 0; sweep < 2; ++sweep) {
    const float2 a = sweep ? make_float2(draw(u0, true), draw(u1, true)) : make_float2(p0, p1);
    const float2 b = sweep ? make_float2(p0, p1) : make_float2(draw(u0, false), draw(u1, false));
    const float2 r = ABS ? x2::pow_abs<F>(a, b) : x2::pow<F>(a, b);
    const float s0 = ABS ? math::pow_abs<F>(a.x, b.x) : math::pow<F>(a.x, b.x);
    const float s1 = ABS ? math::pow_abs<F>(a.y, b.y) : math::pow<F>(a.y, b.y);
    if (!same(r.x, s0)) record(rep, u0);
    if (!same(r.y, s1)) record(rep, u1);
  }
}

// 26, 27: cbrt, unfused and fused
__device__ __forceinline__ void x2_check_cbrt(bool fused, uint32_t u0, x2_report* rep)
{
  const uint32_t u1 = u0 + 1;
  const float2 a = make_float2(__uint_as_float(u0), __uint_as_float(u1));
  const float2 r = fused ? x2::cbrt<true>(a) : x2::cbrt<false>(a);
  const float s0 = fused ? math::cbrt<true>(a.x) : math::cbrt<false>(a.x);
  const float s1 = fused ? math::cbrt<true>(a.y) : math::cbrt<false>(a.y);
  if (!same(r.x, s0)) record(rep, u0);
  if (!same(r.y, s1)) record(rep, u1);
}

__global__ void __launch_bounds__(256) k_x2_check(int which, uint64_t pairs, x2_report* rep)
{
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < pairs; p += (uint64_t)gridDim.x * blockDim.x) {
    if (which < 4) x2_check_pair<false>(which, (uint32_t)(2 * p), rep);
    else if (which < 8) x2_check_pair<true>(which - 4, (uint32_t)(2 * p), rep);
    else if (which < 12) x2_check_fast(which - 8, (uint32_t)(2 * p), rep);
    else if (which == 12) x2_check_fnc<false>((uint32_t)(2 * p), rep);
    else if (which == 13) x2_check_fnc<true>((uint32_t)(2 * p), rep);
    else if (which == 14) x2_check_trig<trig::SIN, false>((uint32_t)(2 * p), rep);
    else if (which == 15) x2_check_trig<trig::COS, false>((uint32_t)(2 * p), rep);
    else if (which == 16) x2_check_trig<trig::SIN, true>((uint32_t)(2 * p), rep);
    else if (which == 17) x2_check_trig<trig::COS, true>((uint32_t)(2 * p), rep);
    else if (which == 18) x2_check_trig<trig::TAN, false>((uint32_t)(2 * p), rep);
    else if (which == 19) x2_check_trig<trig::COT, false>((uint32_t)(2 * p), rep);
    else if (which == 20) x2_check_trig<trig::TAN, true>((uint32_t)(2 * p), rep);
    else if (which == 21) x2_check_trig<trig::COT, true>((uint32_t)(2 * p), rep);
    else if (which == 22) x2_check_pow<false, false>((uint32_t)(2 * p), rep);
    else if (which == 23) x2_check_pow<false, true>((uint32_t)(2 * p), rep);
    else if (which == 24) x2_check_pow<true, false>((uint32_t)(2 * p), rep);
    else if (which == 25) x2_check_pow<true, true>((uint32_t)(2 * p), rep);
    else x2_check_cbrt(which == 27, (uint32_t)(2 * p), rep);
  }
}

}  // namespace

extern "C" nt2cuda_status nt2cuda_selftest_x2(int which, unsigned long long* mismatches, uint32_t* first_bad,
                                              nt2cuda_stream stream)
{
  NT2CUDA_NVTX_RANGE;
  if (which < 0 || which > 27 || !mismatches) return NT2CUDA_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  x2_report* rep = nullptr;
  cudaError_t e = cudaMalloc(&rep, sizeof(x2_report));
  if (e != cudaSuccess) return from_cuda(e);
  e = cudaMemsetAsync(rep, 0, sizeof(x2_report), s);
  if (e == cudaSuccess) {
    const uint64_t pairs = (uint64_t)1 << 31;
    k_x2_check<<<(unsigned)(sm_count() * 8), 256, 0, s>>>(which, pairs, rep);
    e = cudaGetLastError();
  }
  x2_report h{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, rep, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(rep);
  if (e != cudaSuccess) return from_cuda(e);
  *mismatches = h.mismatches;
  if (first_bad)
    for (int i = 0; i < 8; ++i) first_bad[i] = h.first[i];
  return NT2CUDA_OK;
}
