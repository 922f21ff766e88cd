// capi_sigmadelta.cu -- batched sigma-delta background subtraction over many
// uint8 video streams of uneven sizes in one persistent launch.
//
// NT2 runs five separate table assignments per frame
// (demo/sigmadelta/nt2/sigmadelta_nt2.cpp:37-58), each a transform pass over
// the image with the diff and mul temporaries materialised.  Here the five
// statements are fused per pixel, every frame of a stream is processed while
// bkg/var stay in registers, and all streams share one launch driven by a
// (stream, tile) work-list.  Pixels are handled two to a __half2 on the FMA
// pipe (exact small-integer arithmetic); the arithmetic is NT2's:
//   bkg  = selinc(bkg < fr, seldec(bkg > fr, bkg))
//   diff = max(bkg, fr) - min(bkg, fr)
//   mul  = adds(adds(diff, diff), diff)                (saturating uint8)
//   var  = if_else(diff != 0, selinc(var < mul, seldec(var > mul, var)), var)
//   out  = if_zero_else_one(diff < var)
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>
#include "internal.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;

namespace {

constexpr int SD_THREADS = 256;
constexpr int SD_PIX = 16;                          // pixels per thread per tile
constexpr size_t SD_TILE = (size_t)SD_THREADS * SD_PIX;
constexpr int SD_MAX_FRAMES = 64;
constexpr int SD_BATCH = 8;                         // frames whose loads are issued together

struct sd_desc {
  const uint8_t* frames;
  uint64_t frame_stride;
  uint8_t* bkg;
  uint8_t* var;
  uint8_t* labels;
  uint64_t label_stride;
  uint64_t npix;
  uint32_t vec_ok;
  uint32_t pad;
};

// Two pixels per __half2 on the FMA pipe.  Pixel values, their differences,
// 3*diff (<= 765) and the biased values 1024 + x are all integers below 2048,
// so every half-precision operation below is exact.  A byte x becomes the half
// 1024 + x by placing it under the exponent byte 0x64 (one PRMT), and the low
// byte of such a half is x again.
__device__ __forceinline__ void unpack_bytes(uint32_t w, __half2& lo, __half2& hi)
{
  uint32_t a = __byte_perm(w, 0x64646464u, 0x4140);   // [0x64 x1 0x64 x0]
  uint32_t b = __byte_perm(w, 0x64646464u, 0x4342);   // [0x64 x3 0x64 x2]
  lo = *reinterpret_cast<__half2*>(&a);
  hi = *reinterpret_cast<__half2*>(&b);
}

__device__ __forceinline__ uint32_t pack_bytes(__half2 lo, __half2 hi)
{
  uint32_t a = *reinterpret_cast<uint32_t*>(&lo);
  uint32_t b = *reinterpret_cast<uint32_t*>(&hi);
  return __byte_perm(a, b, 0x6420);                  // low bytes of the four halves
}

// One frame step: b and f biased (1024 + x), v plain; returns the biased label.
__device__ __forceinline__ __half2 sd_step_h2(__half2& b, __half2 f, __half2& v)
{
  const __half2 one = __float2half2_rn(1.0f), mone = __float2half2_rn(-1.0f);
  const __half2 zero = __float2half2_rn(0.0f), c255 = __float2half2_rn(255.0f);
  const __half2 three = __float2half2_rn(3.0f);
  const __half2 l1024 = __float2half2_rn(1024.0f);
  b = __hadd2(b, __hmax2(__hmin2(__hsub2(f, b), one), mone));          // bkg one step toward fr
  const __half2 d = __habs2(__hsub2(f, b));                           // |bkg - fr|
  const __half2 m = __hmin2(__hmul2(d, three), c255);                 // adds(adds(d,d),d)
  const __half2 nz = __hmin2(d, one);                                 // d != 0
  v = __hfma2(nz, __hmax2(__hmin2(__hsub2(m, v), one), mone), v);     // var one step toward m
  return __hadd2(__hge2(d, v), l1024);                                // 1024 + (d >= var)
}

__device__ __forceinline__ void sd_step1(uint8_t& b, uint8_t f, uint8_t& v, uint8_t& out)
{
  b = (b < f) ? (uint8_t)(b + 1) : ((b > f) ? (uint8_t)(b - 1) : b);
  uint8_t d = (uint8_t)((b > f ? b : f) - (b < f ? b : f));
  unsigned s3 = 3u * d;
  uint8_t m = (uint8_t)(s3 > 255u ? 255u : s3);
  if (d != 0) v = (v < m) ? (uint8_t)(v + 1) : ((v > m) ? (uint8_t)(v - 1) : v);
  out = (d < v) ? 0 : 1;
}

__global__ void __launch_bounds__(SD_THREADS, 3) k_sigmadelta(const sd_desc* __restrict__ desc,
                                                          const uint64_t* __restrict__ tile_start, int nstreams,
                                                          int nframes, int init)
{
  const uint64_t total = tile_start[nstreams];
  const int first = init ? 1 : 0;
  // Every thread finds its tile's stream itself (same addresses across the
  // block, so the loads are broadcasts served by L1): tiles only move forward,
  // so the search starts from the previous stream and needs no barrier.
  int si = 0;
  for (uint64_t t = blockIdx.x; t < total; t += gridDim.x) {
    if (tile_start[si + 1] <= t) {
      int lo = si + 1, hi = nstreams - 1;      // last stream with tile_start <= t
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tile_start[mid] <= t) lo = mid; else hi = mid - 1;
      }
      si = lo;
    }
    const sd_desc d = desc[si];
    const uint64_t t0 = tile_start[si];
    const uint64_t p = (t - t0) * SD_TILE + (uint64_t)threadIdx.x * SD_PIX;
    if (p >= d.npix) continue;
    if (d.vec_ok && p + SD_PIX <= d.npix) {
      // The state and up to SD_BATCH frames are loaded together (one round
      // trip for the whole batch, 16 bytes x (2 + SD_BATCH) in flight per
      // thread), then the frames are stepped in order and their labels stored.
      const __half2 l1024 = __float2half2_rn(1024.0f);
      int k = first;
      int cnt = (nframes - k < SD_BATCH) ? nframes - k : SD_BATCH;
      uint4 f[SD_BATCH];
      const uint4 wb = __ldcs(reinterpret_cast<const uint4*>((init ? d.frames : d.bkg) + p));
      uint4 wv = make_uint4(0u, 0u, 0u, 0u);
      if (!init) wv = __ldcs(reinterpret_cast<const uint4*>(d.var + p));
#pragma unroll
      for (int q = 0; q < SD_BATCH; ++q)
        if (q < cnt) f[q] = __ldcs(reinterpret_cast<const uint4*>(d.frames + (uint64_t)(k + q) * d.frame_stride + p));
      // state for 16 pixels: 8 biased bkg pairs, 8 var pairs
      __half2 b[8], v[8];
      unpack_bytes(wb.x, b[0], b[1]);
      unpack_bytes(wb.y, b[2], b[3]);
      unpack_bytes(wb.z, b[4], b[5]);
      unpack_bytes(wb.w, b[6], b[7]);
      if (init) {
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = __float2half2_rn(1.0f);
      } else {
        unpack_bytes(wv.x, v[0], v[1]);
        unpack_bytes(wv.y, v[2], v[3]);
        unpack_bytes(wv.z, v[4], v[5]);
        unpack_bytes(wv.w, v[6], v[7]);
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = __hsub2(v[q], l1024);
      }
      for (;;) {
#pragma unroll
        for (int q = 0; q < SD_BATCH; ++q) {
          if (q >= cnt) break;
          const uint32_t fw[4] = {f[q].x, f[q].y, f[q].z, f[q].w};
          uint32_t ow[4];
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            __half2 flo, fhi;
            unpack_bytes(fw[w], flo, fhi);
            const __half2 llo = sd_step_h2(b[2 * w], flo, v[2 * w]);
            const __half2 lhi = sd_step_h2(b[2 * w + 1], fhi, v[2 * w + 1]);
            ow[w] = pack_bytes(llo, lhi);
          }
          __stcs(reinterpret_cast<uint4*>(d.labels + (uint64_t)(k + q - first) * d.label_stride + p),
                 make_uint4(ow[0], ow[1], ow[2], ow[3]));
        }
        k += cnt;
        if (k >= nframes) break;
        cnt = (nframes - k < SD_BATCH) ? nframes - k : SD_BATCH;
#pragma unroll
        for (int q = 0; q < SD_BATCH; ++q)
          if (q < cnt) f[q] = __ldcs(reinterpret_cast<const uint4*>(d.frames + (uint64_t)(k + q) * d.frame_stride + p));
      }
      uint32_t bw[4], vw[4];
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        bw[w] = pack_bytes(b[2 * w], b[2 * w + 1]);
        vw[w] = pack_bytes(__hadd2(v[2 * w], l1024), __hadd2(v[2 * w + 1], l1024));
      }
      __stcs(reinterpret_cast<uint4*>(d.bkg + p), make_uint4(bw[0], bw[1], bw[2], bw[3]));
      __stcs(reinterpret_cast<uint4*>(d.var + p), make_uint4(vw[0], vw[1], vw[2], vw[3]));
    } else {
      const uint64_t end = (p + SD_PIX < d.npix) ? p + SD_PIX : d.npix;
      for (uint64_t q = p; q < end; ++q) {
        uint8_t b, v, o;
        if (init) { b = d.frames[q]; v = 1; } else { b = d.bkg[q]; v = d.var[q]; }
        for (int k = first; k < nframes; ++k) {
          sd_step1(b, d.frames[(uint64_t)k * d.frame_stride + q], v, o);
          d.labels[(uint64_t)(k - first) * d.label_stride + q] = o;
        }
        d.bkg[q] = b;
        d.var[q] = v;
      }
    }
  }
}

struct host_batch {
  std::vector<sd_desc> desc;
  std::vector<uint64_t> tile_start;
};

nt2cuda_status build_batch(const nt2cuda_sd_stream* st, int nstreams, int nframes, int init, host_batch& hb)
{
  if (!st || nstreams <= 0 || nframes <= 0 || nframes > SD_MAX_FRAMES) return NT2CUDA_ERR_ARG;
  if (init && nframes < 2) return NT2CUDA_ERR_ARG;
  hb.desc.resize((size_t)nstreams);
  hb.tile_start.resize((size_t)nstreams + 1);
  uint64_t tiles = 0;
  for (int i = 0; i < nstreams; ++i) {
    const nt2cuda_sd_stream& s = st[i];
    uint64_t npix = (uint64_t)s.width * (uint64_t)s.height;
    if (npix && (!s.frames || !s.bkg || !s.var || !s.labels)) return NT2CUDA_ERR_ARG;
    if (npix && (s.frame_stride < npix || s.label_stride < npix)) return NT2CUDA_ERR_ARG;
    sd_desc d{};
    d.frames = s.frames;
    d.frame_stride = s.frame_stride;
    d.bkg = s.bkg;
    d.var = s.var;
    d.labels = s.labels;
    d.label_stride = s.label_stride;
    d.npix = npix;
    d.vec_ok = ((((uintptr_t)s.frames | (uintptr_t)s.bkg | (uintptr_t)s.var | (uintptr_t)s.labels |
                  (uintptr_t)s.frame_stride | (uintptr_t)s.label_stride) & 15u) == 0) ? 1u : 0u;
    hb.desc[(size_t)i] = d;
    hb.tile_start[(size_t)i] = tiles;
    tiles += (npix + SD_TILE - 1) / SD_TILE;
  }
  hb.tile_start[(size_t)nstreams] = tiles;
  return NT2CUDA_OK;
}

size_t batch_bytes(int nstreams) { return (size_t)nstreams * sizeof(sd_desc) + ((size_t)nstreams + 1) * 8 + 256; }

nt2cuda_status upload_batch(const host_batch& hb, void* dev, cudaStream_t s, sd_desc** d_desc, uint64_t** d_tiles)
{
  size_t db = hb.desc.size() * sizeof(sd_desc);
  size_t off = (db + 255) / 256 * 256;
  *d_desc = (sd_desc*)dev;
  *d_tiles = (uint64_t*)((char*)dev + off);
  cudaError_t e = cudaMemcpyAsync(*d_desc, hb.desc.data(), db, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return from_cuda(e);
  e = cudaMemcpyAsync(*d_tiles, hb.tile_start.data(), hb.tile_start.size() * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return from_cuda(e);
  // the host vectors are pageable: the copies above complete before return
  return NT2CUDA_OK;
}

nt2cuda_status launch_batch(const host_batch& hb, sd_desc* d_desc, uint64_t* d_tiles, int nstreams, int nframes,
                            int init, cudaStream_t s)
{
  uint64_t tiles = hb.tile_start.back();
  if (tiles == 0) return NT2CUDA_OK;
  int per_sm = resident_blocks(k_sigmadelta, SD_THREADS);
  uint64_t grid = (uint64_t)sm_count() * (uint64_t)per_sm;
  if (grid > tiles) grid = tiles;
  k_sigmadelta<<<(unsigned)grid, SD_THREADS, 0, s>>>(d_desc, d_tiles, nstreams, nframes, init);
  return launch_status(cudaSuccess);
}

}  // namespace

struct nt2cuda_sd_plan {
  void* dev = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

nt2cuda_status nt2cuda_sigmadelta_batch_u8(const nt2cuda_sd_stream* streams, int nstreams, int nframes, int init,
                                           nt2cuda_stream stream)
{
  NT2CUDA_NVTX_RANGE;
  host_batch hb;
  nt2cuda_status st = build_batch(streams, nstreams, nframes, init, hb);
  if (st != NT2CUDA_OK) return st;
  cudaStream_t s = as_stream(stream);
  void* dev = nullptr;
  st = detail_capi::stream_scratch(s, batch_bytes(nstreams), &dev, 1);
  if (st != NT2CUDA_OK) return st;
  sd_desc* dd;
  uint64_t* dt;
  st = upload_batch(hb, dev, s, &dd, &dt);
  if (st != NT2CUDA_OK) return st;
  return launch_batch(hb, dd, dt, nstreams, nframes, init, s);
}

nt2cuda_status nt2cuda_sigmadelta_plan_create(const nt2cuda_sd_stream* streams, int nstreams, int nframes, int init,
                                              nt2cuda_stream stream, nt2cuda_sd_plan** plan)
{
  if (!plan) return NT2CUDA_ERR_ARG;
  *plan = nullptr;
  host_batch hb;
  nt2cuda_status st = build_batch(streams, nstreams, nframes, init, hb);
  if (st != NT2CUDA_OK) return st;
  cudaStream_t s = as_stream(stream);
  nt2cuda_sd_plan* p = new nt2cuda_sd_plan();
  cudaError_t e = cudaMalloc(&p->dev, batch_bytes(nstreams));
  if (e != cudaSuccess) { delete p; return from_cuda(e); }
  sd_desc* dd;
  uint64_t* dt;
  st = upload_batch(hb, p->dev, s, &dd, &dt);
  if (st == NT2CUDA_OK) st = from_cuda(cudaStreamSynchronize(s));
  if (st != NT2CUDA_OK) { cudaFree(p->dev); delete p; return st; }
  // capture the launch on a private stream so the caller's stream is never in capture mode
  cudaStream_t cs;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) { cudaFree(p->dev); delete p; return from_cuda(e); }
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    st = launch_batch(hb, dd, dt, nstreams, nframes, init, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &p->graph);
    if (st == NT2CUDA_OK && e2 != cudaSuccess) st = from_cuda(e2);
  } else {
    st = from_cuda(e);
  }
  cudaStreamDestroy(cs);
  if (st == NT2CUDA_OK) st = from_cuda(cudaGraphInstantiate(&p->exec, p->graph, 0));
  if (st != NT2CUDA_OK) {
    if (p->graph) cudaGraphDestroy(p->graph);
    cudaFree(p->dev);
    delete p;
    return st;
  }
  *plan = p;
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_sigmadelta_plan_launch(nt2cuda_sd_plan* plan, nt2cuda_stream stream)
{
  NT2CUDA_NVTX_RANGE;
  if (!plan || !plan->exec) return NT2CUDA_ERR_ARG;
  return from_cuda(cudaGraphLaunch(plan->exec, as_stream(stream)), NT2CUDA_ERR_LAUNCH);
}

nt2cuda_status nt2cuda_sigmadelta_plan_destroy(nt2cuda_sd_plan* plan)
{
  if (!plan) return NT2CUDA_OK;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  if (plan->dev) cudaFree(plan->dev);
  delete plan;
  return NT2CUDA_OK;
}

}  // extern "C"
