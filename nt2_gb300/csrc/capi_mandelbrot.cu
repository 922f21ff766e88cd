// capi_mandelbrot.cu -- the mandelbrot demo's arrayfun on the GPU.
//
// NT2 evaluates C = arrayfun(step, A, B) (demo/mandelbrot/nt2/mandelbrot_nt2.cpp:120-123)
// with its transform skeleton: the step functor runs on SIMD packs of
// consecutive elements, then on single elements for the n % N tail
// (modules/core/base/include/nt2/core/functions/simd/transform.hpp:40-57).
// The functor (mandelbrot_nt2.cpp:55-81) iterates z <- z^2 + c for the
// whole pack until no lane satisfies |z|^2 < 4 or 256 trips are done,
// adding 1 to a lane's count on each trip where its |z|^2 (taken before the
// update) was below 4.
//
// Here one thread owns one element and a pack is a group of `PACK`
// consecutive lanes of a warp: one ballot per trip gives each group its
// any(mask).  Elements are independent; the kernel is bound by FP32 issue
// (seven rounded operations, a compare, a count and a vote per trip).
// Every operation is an IEEE `__f*_rn` call, so nothing is contracted and
// the counts equal the scalar CPU evaluation bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;

namespace {

constexpr int kTrips = 256;   // mandelbrot_nt2.cpp:79, `while(flag && i < 256)`

// Coordinates of the demo's program: A(i,j) = linspace(a0,a1,w)(j),
// B(i,j) = linspace(b0,b1,h)(i) for the column-major element e = i + j*h.
struct grid {
  float a0, a1, sa, b0, b1, sb;
  uint64_t h, w;
};

// linspace(lo,hi,n)(p): hi at p = n-1, else fma(p, step, lo) with NT2's
// generic (unfused) fma (nt2/core/functions/details/linspace.hpp:33-45).
__device__ __forceinline__ float lin(float lo, float step, float hi, uint64_t last, uint64_t p)
{
  return p == last ? hi : __fadd_rn(__fmul_rn((float)p, step), lo);
}

template <int PACK, bool GRID>
__global__ void __launch_bounds__(256) k_mandelbrot(const float* __restrict__ A, const float* __restrict__ B,
                                                    grid gr, int32_t* __restrict__ C, uint64_t n,
                                                    uint64_t nfull)
{
  nt2cuda::mem::pdl_begin();
  const uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  const bool in = e < n;
  float a = 0.f, b = 0.f;
  if (in) {
    if constexpr (GRID) {
      const uint64_t i = e % gr.h, j = e / gr.h;
      a = lin(gr.a0, gr.sa, gr.a1, gr.w - 1, j);
      b = lin(gr.b0, gr.sb, gr.b1, gr.h - 1, i);
    } else {
      a = A[e];
      b = B[e];
    }
  }
  // lanes of this element's pack; elements past the last whole pack are alone
  unsigned seg = 1u << lane;
  if (PACK > 1 && e < nfull)
    seg = (PACK == 32 ? 0xffffffffu : ((1u << PACK) - 1u)) << (lane & ~(unsigned)(PACK - 1));
  bool alive = in;
  int32_t iter = 0;
  float x = 0.f, y = 0.f;
  unsigned live = __ballot_sync(0xffffffffu, alive);
#pragma unroll 1
  for (int t = 0; t < kTrips && live; ++t) {
    const float x2 = __fmul_rn(x, x);
    const float y2 = __fmul_rn(y, y);
    const float xy = __fmul_rn(__fmul_rn(2.f, x), y);
    x = __fadd_rn(__fsub_rn(x2, y2), a);
    y = __fadd_rn(xy, b);
    const bool mask = alive && __fadd_rn(x2, y2) < 4.f;
    iter += mask ? 1 : 0;
    // a pack goes on while any of its lanes' masks held (mask implies alive)
    live = __ballot_sync(0xffffffffu, mask);
    alive = (live & seg) != 0u;
  }
  if (in) C[e] = iter;
}

template <bool GRID>
nt2cuda_status launch(const float* A, const float* B, const grid& g, int32_t* C, uint64_t n, int pack,
                      cudaStream_t s)
{
  if (!n) return NT2CUDA_OK;
  const uint64_t nfull = n - n % (uint64_t)pack;
  const uint64_t blocks = (n + 255) / 256;
  if (blocks > 0x7fffffffULL) return NT2CUDA_ERR_ARG;
  void* args[] = {(void*)&A, (void*)&B, (void*)&g, (void*)&C, (void*)&n, (void*)&nfull};
  cudaError_t e;
  switch (pack) {
    case 1: e = launch_grid(k_mandelbrot<1, GRID>, blocks, 256, s, args); break;
    case 2: e = launch_grid(k_mandelbrot<2, GRID>, blocks, 256, s, args); break;
    case 4: e = launch_grid(k_mandelbrot<4, GRID>, blocks, 256, s, args); break;
    case 8: e = launch_grid(k_mandelbrot<8, GRID>, blocks, 256, s, args); break;
    case 16: e = launch_grid(k_mandelbrot<16, GRID>, blocks, 256, s, args); break;
    case 32: e = launch_grid(k_mandelbrot<32, GRID>, blocks, 256, s, args); break;
    default: return NT2CUDA_ERR_ARG;
  }
  if (e != cudaSuccess) return launch_status(e);
  return launch_status(cudaGetLastError());
}

bool pack_ok(int pack) { return pack == 1 || pack == 2 || pack == 4 || pack == 8 || pack == 16 || pack == 32; }

}  // namespace

extern "C" {

nt2cuda_status nt2cuda_mandelbrot_f32(const float* A, const float* B, int32_t* C, size_t n, int pack,
                                      nt2cuda_stream stream)
{
  NT2CUDA_NVTX_RANGE;
  if (!pack_ok(pack) || (n && (!A || !B || !C))) return NT2CUDA_ERR_ARG;
  const uintptr_t c0 = (uintptr_t)C, c1 = c0 + n * 4;
  for (const float* p : {A, B}) {
    const uintptr_t p0 = (uintptr_t)p, p1 = p0 + n * 4;
    if (n && p0 < c1 && c0 < p1) return NT2CUDA_ERR_ALIAS;
  }
  return launch<false>(A, B, grid{}, C, (uint64_t)n, pack, as_stream(stream));
}

nt2cuda_status nt2cuda_mandelbrot_grid_f32(float a0, float a1, float b0, float b1, size_t h, size_t w,
                                           int32_t* C, int pack, nt2cuda_stream stream)
{
  NT2CUDA_NVTX_RANGE;
  if (!pack_ok(pack) || (h && w && !C)) return NT2CUDA_ERR_ARG;
  if (!h || !w) return NT2CUDA_OK;
  grid g{};
  g.a0 = a0; g.a1 = a1; g.b0 = b0; g.b1 = b1; g.h = h; g.w = w;
  // step = (u - l) / real_type(n - 1), computed once in float as NT2 does (linspace.hpp:27-31)
  g.sa = (a1 - a0) / (float)(w - 1);
  g.sb = (b1 - b0) / (float)(h - 1);
  return launch<true>(nullptr, nullptr, g, C, (uint64_t)h * (uint64_t)w, pack, as_stream(stream));
}

}  // extern "C"
