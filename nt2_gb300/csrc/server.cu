// server.cu -- continuous-batching request loop for Black-Scholes pricing
// requests of mixed sizes.
//
// NT2 has no serving layer; every evaluation is one synchronous statement on
// the calling thread.  This server accepts requests whose inputs are already
// resident in HBM, keeps their outputs resident in a device arena admitted
// against a memory budget, and coalesces whatever requests are admitted at
// each step into one launch over a (request, tile) work-list.  Up to
// max_inflight_batches launches are on the device at once (one stream each),
// so requests that arrive while a batch runs are admitted and launched
// without waiting for it.  All waiting of these two modes happens on the
// host with bounded waits.  The resident mode (below) keeps one kernel on
// the device instead; its waits are bounded in time.
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <cstring>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>
#include "internal.cuh"
#include "nt2cuda/blackscholes.cuh"
#include "nt2cuda/launch.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;

namespace {

using clk = std::chrono::steady_clock;
inline uint64_t now_ns()
{
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(clk::now().time_since_epoch()).count();
}

constexpr size_t BS_TILE = 256 * 4 * 2;   // options per work-list tile (2 groups of 4 per thread)

struct req_desc {
  const float* S;
  const float* K;
  const float* T;
  float* call;
  float* put;
  uint64_t n;
  float r, sigma;
  uint32_t vec_ok;
  uint32_t pad;
};

// Small batches travel in the kernel's parameter block (no descriptor copy
// before the launch); larger ones in a device buffer filled by one copy.
constexpr int kInline = 16;
struct inline_list {
  req_desc d[kInline];
  uint64_t tile_start[kInline + 1];
};

// One launch over all requests of a batch.  Each block takes tiles from the
// work-list; tile_start[i] is the first tile of request i.  The per-option
// arithmetic is bs_lane, the same function the single-request kernel uses,
// so a request's results do not depend on what it was batched with.
// Options [base, base + BS_TILE) of one request, by the whole block.
template <int CDF, int P>
__device__ __forceinline__ void bs_tile(const req_desc& d, uint64_t base)
{
  const float c = math::madd<(P != PREC_EXACT)>(math::mul(d.sigma, d.sigma), 0.5f, d.r);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint64_t i = base + (uint64_t)h * 1024 + (uint64_t)threadIdx.x * 4;
    if (i >= d.n) continue;
    if (d.vec_ok && i + 4 <= d.n) {
      float s[4], k[4], tt[4], oc[4], op[4];
      mem::load_vec<float, 4, true>(d.S, i, s);
      mem::load_vec<float, 4, true>(d.K, i, k);
      mem::load_vec<float, 4, true>(d.T, i, tt);
      if constexpr (kPacked<float, CDF, P> || kPackedFast<float, CDF, P>) {
#pragma unroll
        for (int l = 0; l < 4; l += 2) {
          float2 pc, pp;
          const float2 ps = make_float2(s[l], s[l + 1]), pk = make_float2(k[l], k[l + 1]),
                       pt = make_float2(tt[l], tt[l + 1]);
          if constexpr (kPackedFast<float, CDF, P>) x2::fast::blackscholes(ps, pk, pt, d.r, d.sigma, c, pc, pp);
          else if constexpr (CDF == CDF_FASTNORMCDF)
            x2::blackscholes_fastnormcdf<P == PREC_FUSED>(ps, pk, pt, d.r, d.sigma, c, pc, pp);
          else x2::blackscholes<P == PREC_FUSED>(ps, pk, pt, d.r, d.sigma, c, pc, pp);
          oc[l] = pc.x; oc[l + 1] = pc.y;
          op[l] = pp.x; op[l + 1] = pp.y;
        }
      } else {
#pragma unroll
        for (int l = 0; l < 4; ++l) bs_lane<float, CDF, P>(s[l], k[l], tt[l], d.r, d.sigma, c, oc[l], op[l]);
      }
      mem::store_vec<float, 4>(d.call, i, oc);
      mem::store_vec<float, 4>(d.put, i, op);
    } else {
      const uint64_t e = (i + 4 < d.n) ? i + 4 : d.n;
      for (uint64_t q = i; q < e; ++q)
        bs_lane<float, CDF, P>(d.S[q], d.K[q], d.T[q], d.r, d.sigma, c, d.call[q], d.put[q]);
    }
  }
}

template <int CDF, int P>
__device__ __forceinline__ void bs_batch_body(const req_desc* desc, const uint64_t* tile_start, int nreq)
{
  __shared__ int s_req;
  const uint64_t total = tile_start[nreq];
  for (uint64_t t = blockIdx.x; t < total; t += gridDim.x) {
    if (threadIdx.x == 0) {
      int lo = 0, hi = nreq - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tile_start[mid] <= t) lo = mid; else hi = mid - 1;
      }
      s_req = lo;
    }
    __syncthreads();
    const int ri = s_req;
    const req_desc d = desc[ri];
    const uint64_t t0 = tile_start[ri];
    __syncthreads();
    bs_tile<CDF, P>(d, (t - t0) * BS_TILE);
  }
}

template <int CDF, int P>
__global__ void __launch_bounds__(256) k_bs_batch(const req_desc* __restrict__ desc,
                                                  const uint64_t* __restrict__ tile_start, int nreq)
{
  bs_batch_body<CDF, P>(desc, tile_start, nreq);
}

template <int CDF, int P>
__global__ void __launch_bounds__(256) k_bs_batch_inline(const __grid_constant__ inline_list list, int nreq)
{
  bs_batch_body<CDF, P>(list.d, list.tile_start, nreq);
}

// ------------------------------------------------------- resident mode
// coalesce = 2: one kernel stays on the device and drains a ring of requests
// that the host publishes in pinned, device-mapped memory, so a request that
// arrives while others run joins the running kernel instead of waiting for a
// launch.  Block 0 is the manager: it copies newly published ring entries
// into device memory and publishes their tiles.  Every other block takes a
// tile ticket (one atomic add on the next-tile counter) and, once that tile
// is published, prices it with the batch kernel's arithmetic; the block that
// finishes a request's last tile writes the request's completion word in host
// memory.  Every wait is bounded in time (%globaltimer): the manager leaves
// after idle_ns without new requests once every published tile is finished,
// or after stall_ns without a finished tile while tiles wait (the workers are
// gone); a block whose wait for its tile exceeds its own bound records an
// error and leaves.  The host launches the kernel again when a request is published
// after it left.
constexpr uint32_t kRing = 4096;            // requests published and not yet complete, at most

struct ring_entry {
  req_desc d;
  uint64_t tile_begin, ntiles, seq, pad;
};

enum : uint32_t { RES_RUNNING = 0, RES_IDLE_EXIT = 1, RES_STOPPED = 2, RES_WAIT_TIMEOUT = 3 };

// pinned host memory mapped into the device's address space
struct resident_host {
  ring_entry ring[kRing];                   // written by the host
  uint64_t tail;                            // requests published (host, store-release)
  uint32_t stop;                            // host: leave once drained
  uint32_t status;                          // kernel: why it left
  uint64_t consumed;                        // kernel: requests copied when it left
  uint64_t done[kRing];                     // kernel: seq + 1 once request seq is complete
};

// device memory, kept across launches; the counters every block touches sit
// on 128-byte lines of their own
struct __align__(128) resident_line { uint64_t v; uint64_t pad[15]; };
struct resident_dev {
  ring_entry ring[kRing];
  resident_line nreq;                       // requests copied
  resident_line pub;                        // end of the published tiles
  resident_line next;                       // next tile ticket (may run ahead of pub)
  resident_line processed;                  // tiles finished
  resident_line closing;                    // 1: no tile will be published any more
  uint32_t error;
  unsigned tiles_done[kRing];
};

__device__ __forceinline__ uint64_t gtimer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ uint64_t ld_acq_sys(const uint64_t* p)
{
  uint64_t v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acq_sys32(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t ld_acq_gpu(const uint64_t* p)
{
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acq_gpu32(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_rel_gpu(uint64_t* p, uint64_t v)
{
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rel_gpu32(uint32_t* p, uint32_t v)
{
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_rel_sys(uint64_t* p, uint64_t v)
{
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rel_sys32(uint32_t* p, uint32_t v)
{
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// A ring entry read past the L1 cache (ld.cv: fetched again on every read):
// its slot was written by another agent (the host, or the manager) after
// this SM may have cached the slot's previous occupant.
__device__ __forceinline__ ring_entry load_entry_cv(const ring_entry* p)
{
  ring_entry e;
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(p);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&e);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(ring_entry) / 8); ++i) dst[i] = __ldcv(src + i);
  return e;
}
__device__ __forceinline__ ring_entry load_entry_cg(const ring_entry* p)
{
  ring_entry e;
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(p);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&e);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(ring_entry) / 8); ++i) dst[i] = __ldcg(src + i);
  return e;
}

__device__ void resident_manager(resident_host* h, resident_dev* d, uint64_t idle_ns)
{
  uint64_t copied = d->nreq.v;
  uint64_t last = gtimer();                                       // last new request
  uint64_t seen = ld_acq_gpu(&d->processed.v), moved = last;      // last tile finished
  uint32_t reason = RES_IDLE_EXIT;
  // published tiles that none finishes for this long mean the workers are gone
  const uint64_t stall_ns = 4 * idle_ns + 1000000000ull;
  for (;;) {
    const uint64_t tail = ld_acq_sys(&h->tail);
    if (tail > copied) {
      const uint64_t end = (tail - copied > 64) ? copied + 64 : tail;
      uint64_t pub_end = 0;
      for (uint64_t i = copied; i < end; ++i) {
        const ring_entry e = load_entry_cv(&h->ring[i % kRing]);
        d->ring[i % kRing] = e;
        d->tiles_done[i % kRing] = 0u;
        pub_end = e.tile_begin + e.ntiles;
      }
      d->nreq.v = end;
      __threadfence();                                            // the entries and counters before the tiles
      st_rel_gpu(&d->pub.v, pub_end);
      copied = end;
      last = gtimer();
      continue;
    }
    const uint64_t now = gtimer();
    const uint64_t done = ld_acq_gpu(&d->processed.v);
    const bool drained = done >= ld_acq_gpu(&d->pub.v);
    if (done != seen) { seen = done; moved = now; }
    if (drained && ld_acq_sys32(&h->stop)) { reason = RES_STOPPED; break; }
    if (drained && now - last > idle_ns) break;
    if (!drained && now - moved > stall_ns) { reason = RES_WAIT_TIMEOUT; break; }
    __nanosleep(256);
  }
  st_rel_gpu(&d->closing.v, 1u);
  h->consumed = copied;
  __threadfence_system();
  st_rel_sys32(&h->status, reason);
}

template <int CDF, int P>
__global__ void __launch_bounds__(256) k_bs_resident(resident_host* h, resident_dev* d, uint64_t idle_ns,
                                                     uint64_t first_req)
{
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) resident_manager(h, d, idle_ns);
    return;
  }
  __shared__ uint64_t s_tile, s_cursor;
  __shared__ ring_entry s_e;
  uint64_t cursor = first_req;
  // a wait for work outlives the manager's idle bound only if the manager is gone
  const uint64_t wait_ns = 2 * idle_ns + 100000000ull;
  for (;;) {
    if (threadIdx.x == 0) {
      // a ticket always succeeds; it may name a tile not published yet, which
      // the block waits for (the next request's first tiles go to the blocks
      // already waiting, in ticket order)
      uint64_t tile = atomicAdd((unsigned long long*)&d->next.v, 1ull);
      const uint64_t t0 = gtimer();
      unsigned nap = 64;
      for (;;) {
        if (tile < ld_acq_gpu(&d->pub.v)) break;
        if (ld_acq_gpu(&d->closing.v)) { tile = ~0ull; break; }   // nothing more will be published
        if (gtimer() - t0 > wait_ns) {
          atomicExch(&d->error, 1u);
          st_rel_sys32(&h->status, RES_WAIT_TIMEOUT);
          tile = ~0ull;
          break;
        }
        __nanosleep(nap);
        if (nap < 1024) nap <<= 1;
      }
      if (tile != ~0ull) {
        // the request holding this tile: scan forward from the last one (a ring
        // slot whose seq moved on belongs to a later request: this one is done);
        // every request up to the one holding the tile is already copied, so the
        // scan ends before d->nreq, or the ring is corrupt and the block leaves
        const uint64_t nreq = ld_acq_gpu(&d->nreq.v);
        ring_entry e = load_entry_cg(&d->ring[cursor % kRing]);
        while (!(e.seq == cursor && tile < e.tile_begin + e.ntiles) && cursor < nreq) {
          ++cursor;
          e = load_entry_cg(&d->ring[cursor % kRing]);
        }
        if (cursor >= nreq) {
          atomicExch(&d->error, 2u);
          st_rel_sys32(&h->status, RES_WAIT_TIMEOUT);
          tile = ~0ull;
        } else {
          s_e = e;
          s_cursor = cursor;
        }
      }
      s_tile = tile;
    }
    __syncthreads();
    const uint64_t tile = s_tile;
    if (tile == ~0ull) return;
    const ring_entry e = s_e;
    bs_tile<CDF, P>(e.d, (tile - e.tile_begin) * BS_TILE);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      const unsigned prev = atomicAdd(&d->tiles_done[s_cursor % kRing], 1u);
      if (prev + 1u == (unsigned)e.ntiles) {
        __threadfence_system();                                  // the request's prices before its completion word
        st_rel_sys(&h->done[s_cursor % kRing], e.seq + 1);
      }
      atomicAdd((unsigned long long*)&d->processed.v, 1ull);
    }
    __syncthreads();
  }
}

// Persistent grid of a batch kernel: resident blocks per SM x SMs, computed
// once per instantiation (this also loads the kernel, so the first request
// does not pay for lazy module loading).
template <class K> int batch_grid(K kernel)
{
  static const int g = sm_count() * resident_blocks(kernel, 256);
  return g;
}

// ------------------------------------------------------- device arena
// First-fit allocator over one cudaMalloc'd region; offsets are 256-aligned.
class arena {
 public:
  bool init(size_t bytes)
  {
    cap_ = bytes;
    if (cudaMalloc(&base_, bytes) != cudaSuccess) { base_ = nullptr; return false; }
    free_[0] = bytes;
    return true;
  }
  ~arena() { if (base_) cudaFree(base_); }
  bool alloc(size_t bytes, size_t* off)
  {
    bytes = (bytes + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        size_t rest = it->second - bytes, o = it->first + bytes;
        free_.erase(it);
        if (rest) free_[o] = rest;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes)
  {
    bytes = (bytes + 255) / 256 * 256;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
    }
  }
  char* ptr(size_t off) const { return (char*)base_ + off; }
  size_t capacity() const { return cap_; }

 private:
  void* base_ = nullptr;
  size_t cap_ = 0;
  std::map<size_t, size_t> free_;
};

enum req_state { WAITING = 0, ADMITTED = 1, LAUNCHED = 2, DONE = 3 };

struct request {
  uint64_t id;
  req_desc d;
  size_t off = 0, bytes = 0;
  int state = WAITING;
  uint64_t t_submit = 0, t_done = 0;
};

struct batch;

// One launch slot: a stream, an event, and the work-list of the batch it
// carries (descriptors then tile starts, in one pinned buffer copied to the
// device in one transfer).
struct slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  char* h_buf = nullptr;          // pinned
  char* d_buf = nullptr;
  req_desc* h_desc = nullptr;
  uint64_t* h_tiles = nullptr;
  req_desc* d_desc = nullptr;
  uint64_t* d_tiles = nullptr;
  size_t bytes = 0;
  bool busy = false;
};

}  // namespace

struct nt2cuda_server {
  nt2cuda_server_config cfg;
  int device = 0;
  arena mem;
  std::mutex m;
  std::condition_variable cv_work;   // worker: new admitted requests or stop
  std::condition_variable cv_done;   // clients: completions, freed slots, freed memory
  std::unordered_map<uint64_t, request> reqs;
  std::deque<uint64_t> waiting;      // submitted, not yet admitted (budget)
  std::deque<uint64_t> admitted;     // admitted, not yet launched
  std::vector<slot> slots;
  uint64_t next_id = 1;
  size_t reserved = 0;
  bool stop = false;
  std::thread worker;
  std::thread reaper;
  std::deque<struct batch*> inflight;   // launched batches, in launch order
  std::condition_variable cv_inflight;  // reaper: a batch was launched or stop
  nt2cuda_server_stats st{};
  nt2cuda_status worker_error = NT2CUDA_OK;
  std::atomic<int> n_admitted{0};    // admitted.size(), readable without the lock
  uint64_t spin_ns = 0;
  // resident mode (coalesce = 2)
  resident_host* rh = nullptr;       // pinned, mapped
  resident_host* rh_dev = nullptr;   // its device address
  resident_dev* rd = nullptr;
  cudaStream_t rstream = nullptr;
  bool rrunning = false;             // a resident kernel was launched and has not been seen to finish
  uint64_t rseq = 0;                 // requests published
  uint64_t rtiles = 0;               // tiles published
  uint64_t rfirst = 0;               // first request of the running kernel
  int rgrid = 0;
  std::deque<std::pair<uint64_t, uint64_t>> rpending;   // (seq, request id) published, not seen complete
};

namespace {

struct batch {
  nt2cuda_server* srv;
  int slot;
  std::vector<uint64_t> ids;
};

void admit_locked(nt2cuda_server* s)
{
  while (!s->waiting.empty()) {
    request& r = s->reqs[s->waiting.front()];
    size_t off;
    if (s->reserved + r.bytes > s->cfg.budget_bytes || !s->mem.alloc(r.bytes, &off)) break;
    r.off = off;
    r.d.call = (float*)s->mem.ptr(off);
    r.d.put = (float*)s->mem.ptr(off + (r.bytes / 2));
    r.state = ADMITTED;
    s->reserved += r.bytes;
    s->st.reserved_bytes = s->reserved;
    if (s->reserved > s->st.peak_reserved_bytes) s->st.peak_reserved_bytes = s->reserved;
    s->admitted.push_back(r.id);
    s->n_admitted.store((int)s->admitted.size(), std::memory_order_release);
    s->waiting.pop_front();
  }
}

// Completion: the reaper waits for each launched batch's event in launch
// order, stamps its requests done and frees its slot.
void complete_batch(nt2cuda_server* s, batch* b, cudaError_t err)
{
  uint64_t t = now_ns();
  {
    std::lock_guard<std::mutex> g(s->m);
    for (uint64_t id : b->ids) {
      auto it = s->reqs.find(id);
      if (it == s->reqs.end()) continue;
      it->second.state = DONE;
      it->second.t_done = t;
      s->st.completed++;
    }
    if (err != cudaSuccess && s->worker_error == NT2CUDA_OK) s->worker_error = from_cuda(err, NT2CUDA_ERR_LAUNCH);
    s->slots[(size_t)b->slot].busy = false;
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();
  delete b;
}

void reaper_loop(nt2cuda_server* s)
{
  cudaSetDevice(s->device);
  for (;;) {
    batch* b = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->m);
      s->cv_inflight.wait(lk, [&] { return s->stop || !s->inflight.empty(); });
      if (s->inflight.empty()) return;   // stop requested and nothing left
      b = s->inflight.front();
      s->inflight.pop_front();
    }
    cudaError_t e = cudaEventSynchronize(s->slots[(size_t)b->slot].done);
    complete_batch(s, b, e);
  }
}

template <int CDF, int P>
nt2cuda_status launch_batch(nt2cuda_server* s, slot& sl, int nreq)
{
  uint64_t tiles = sl.h_tiles[nreq];
  if (nreq <= kInline) {
    inline_list list;
    for (int i = 0; i < nreq; ++i) { list.d[i] = sl.h_desc[i]; list.tile_start[i] = sl.h_tiles[i]; }
    list.tile_start[nreq] = tiles;
    uint64_t grid = (uint64_t)batch_grid(k_bs_batch_inline<CDF, P>);
    if (grid > tiles) grid = tiles;
    if (grid < 1) grid = 1;
    k_bs_batch_inline<CDF, P><<<(unsigned)grid, 256, 0, sl.stream>>>(list, nreq);
    (void)s;
    return launch_status(cudaGetLastError());
  }
  // descriptors [0, nreq) and tile starts [0, nreq] sit at fixed offsets of one buffer
  const size_t used = (size_t)((char*)(sl.h_tiles + nreq + 1) - sl.h_buf);
  cudaError_t e = cudaMemcpyAsync(sl.d_buf, sl.h_buf, used, cudaMemcpyHostToDevice, sl.stream);
  if (e != cudaSuccess) return from_cuda(e);
  uint64_t grid = (uint64_t)batch_grid(k_bs_batch<CDF, P>);
  if (grid > tiles) grid = tiles;
  if (grid < 1) grid = 1;
  k_bs_batch<CDF, P><<<(unsigned)grid, 256, 0, sl.stream>>>(sl.d_desc, sl.d_tiles, nreq);
  return launch_status(cudaGetLastError());
}

// Load (and size) the kernels this server will launch before the first request.
template <int CDF, int P> void warm_batch()
{
  (void)batch_grid(k_bs_batch_inline<CDF, P>);
  (void)batch_grid(k_bs_batch<CDF, P>);
}

void warm(const nt2cuda_server_config& c)
{
  if (c.coalesce) {
    if (c.cdf_kind == CDF_FASTNORMCDF)
      c.fused == PREC_FAST ? warm_batch<CDF_FASTNORMCDF, PREC_FAST>()
      : c.fused == PREC_FUSED ? warm_batch<CDF_FASTNORMCDF, PREC_FUSED>() : warm_batch<CDF_FASTNORMCDF, PREC_EXACT>();
    else
      c.fused == PREC_FAST ? warm_batch<CDF_NORMCDF, PREC_FAST>()
      : c.fused == PREC_FUSED ? warm_batch<CDF_NORMCDF, PREC_FUSED>() : warm_batch<CDF_NORMCDF, PREC_EXACT>();
  } else {
    warm_blackscholes_f32(c.cdf_kind, c.fused);
  }
}

nt2cuda_status launch_single(nt2cuda_server* s, slot& sl, const req_desc& d)
{
  int cdf = s->cfg.cdf_kind, fused = s->cfg.fused;
  // one launch per request: the plain single-statement entry point
  return nt2cuda_blackscholes_f32(d.S, d.K, d.T, d.r, d.sigma, d.call, d.put, (size_t)d.n, cdf, fused,
                                  reinterpret_cast<nt2cuda_stream>(sl.stream));
}

void worker_loop(nt2cuda_server* s)
{
  cudaSetDevice(s->device);
  const int maxb = s->cfg.coalesce ? std::max(1, s->cfg.max_batch_requests) : 1;
  for (;;) {
    // poll briefly before sleeping: a request that arrives within spin_ns is
    // launched without waiting for the thread to be woken
    if (s->spin_ns && s->n_admitted.load(std::memory_order_acquire) == 0) {
      const uint64_t until = now_ns() + s->spin_ns;
      while (s->n_admitted.load(std::memory_order_acquire) == 0 && now_ns() < until) {
      }
    }
    std::unique_lock<std::mutex> lk(s->m);
    int si = -1;
    s->cv_work.wait(lk, [&] {
      if (s->stop) return true;
      if (s->admitted.empty()) return false;
      for (size_t i = 0; i < s->slots.size(); ++i)
        if (!s->slots[i].busy) { si = (int)i; return true; }
      return false;
    });
    if (s->stop) return;
    slot& sl = s->slots[(size_t)si];
    batch* b = new batch{s, si, {}};
    int nreq = 0;
    uint64_t tiles = 0;
    while (!s->admitted.empty() && nreq < maxb) {
      request& r = s->reqs[s->admitted.front()];
      s->admitted.pop_front();
      r.state = LAUNCHED;
      sl.h_desc[nreq] = r.d;
      sl.h_tiles[nreq] = tiles;
      tiles += (r.d.n + BS_TILE - 1) / BS_TILE;
      b->ids.push_back(r.id);
      ++nreq;
    }
    s->n_admitted.store((int)s->admitted.size(), std::memory_order_release);
    sl.h_tiles[nreq] = tiles;
    sl.busy = true;
    s->st.batches++;
    lk.unlock();

    nt2cuda_status rs = NT2CUDA_OK;
    if (s->cfg.coalesce) {
      const int P = s->cfg.fused;
      if (s->cfg.cdf_kind == CDF_FASTNORMCDF)
        rs = P == PREC_FAST ? launch_batch<CDF_FASTNORMCDF, PREC_FAST>(s, sl, nreq)
           : P == PREC_FUSED ? launch_batch<CDF_FASTNORMCDF, PREC_FUSED>(s, sl, nreq)
                             : launch_batch<CDF_FASTNORMCDF, PREC_EXACT>(s, sl, nreq);
      else
        rs = P == PREC_FAST ? launch_batch<CDF_NORMCDF, PREC_FAST>(s, sl, nreq)
           : P == PREC_FUSED ? launch_batch<CDF_NORMCDF, PREC_FUSED>(s, sl, nreq)
                             : launch_batch<CDF_NORMCDF, PREC_EXACT>(s, sl, nreq);
      lk.lock();
      s->st.launches++;
      lk.unlock();
    } else {
      for (int i = 0; i < nreq && rs == NT2CUDA_OK; ++i) rs = launch_single(s, sl, sl.h_desc[i]);
      lk.lock();
      s->st.launches += (uint64_t)nreq;
      lk.unlock();
    }
    if (rs == NT2CUDA_OK) rs = from_cuda(cudaEventRecord(sl.done, sl.stream));
    if (rs != NT2CUDA_OK) {
      lk.lock();
      s->worker_error = rs;
      for (uint64_t id : b->ids) { request& r = s->reqs[id]; r.state = DONE; r.t_done = now_ns(); }
      sl.busy = false;
      lk.unlock();
      s->cv_done.notify_all();
      delete b;
      continue;
    }
    lk.lock();
    s->inflight.push_back(b);
    lk.unlock();
    s->cv_inflight.notify_one();
  }
}

// ---------------------------------------------------- resident mode, host
constexpr uint64_t kResidentIdleNs = 20000000ull;   // the kernel leaves after 20 ms without requests

template <int CDF, int P> cudaError_t launch_resident_t(nt2cuda_server* s)
{
  k_bs_resident<CDF, P><<<(unsigned)s->rgrid, 256, 0, s->rstream>>>(s->rh_dev, s->rd, kResidentIdleNs, s->rfirst);
  return cudaGetLastError();
}
cudaError_t launch_resident(nt2cuda_server* s)
{
  const int P = s->cfg.fused;
  if (s->cfg.cdf_kind == CDF_FASTNORMCDF)
    return P == PREC_FAST ? launch_resident_t<CDF_FASTNORMCDF, PREC_FAST>(s)
         : P == PREC_FUSED ? launch_resident_t<CDF_FASTNORMCDF, PREC_FUSED>(s)
                           : launch_resident_t<CDF_FASTNORMCDF, PREC_EXACT>(s);
  return P == PREC_FAST ? launch_resident_t<CDF_NORMCDF, PREC_FAST>(s)
       : P == PREC_FUSED ? launch_resident_t<CDF_NORMCDF, PREC_FUSED>(s)
                         : launch_resident_t<CDF_NORMCDF, PREC_EXACT>(s);
}
template <int CDF, int P> int resident_grid_t()
{
  // the manager and the workers all resident at once, one block per SM
  // below full occupancy so that other streams' kernels still find room
  const int per = resident_blocks(k_bs_resident<CDF, P>, 256);
  return sm_count() * (per > 1 ? per - 1 : 1) + 1;
}
int resident_grid(const nt2cuda_server_config& c)
{
  const int P = c.fused;
  if (c.cdf_kind == CDF_FASTNORMCDF)
    return P == PREC_FAST ? resident_grid_t<CDF_FASTNORMCDF, PREC_FAST>()
         : P == PREC_FUSED ? resident_grid_t<CDF_FASTNORMCDF, PREC_FUSED>() : resident_grid_t<CDF_FASTNORMCDF, PREC_EXACT>();
  return P == PREC_FAST ? resident_grid_t<CDF_NORMCDF, PREC_FAST>()
       : P == PREC_FUSED ? resident_grid_t<CDF_NORMCDF, PREC_FUSED>() : resident_grid_t<CDF_NORMCDF, PREC_EXACT>();
}

// The resident-mode thread: publishes admitted requests to the ring, keeps a
// kernel running while requests are outstanding, and marks requests done as
// their completion words appear.
void resident_loop(nt2cuda_server* s)
{
  cudaSetDevice(s->device);
  uint64_t idle_since = now_ns();
  for (;;) {
    bool active = false;
    uint64_t published = 0;
    {
      std::unique_lock<std::mutex> lk(s->m);
      if (s->stop && s->rpending.empty()) break;      // published requests finish; the rest are dropped
      bool any = false;
      while (!s->stop && !s->admitted.empty()) {
        const uint64_t seq = s->rseq;
        const uint32_t slot = (uint32_t)(seq % kRing);
        if (seq >= kRing && __atomic_load_n(&s->rh->done[slot], __ATOMIC_ACQUIRE) != seq - kRing + 1) break;
        request& r = s->reqs[s->admitted.front()];
        s->admitted.pop_front();
        const uint64_t ntiles = (r.d.n + BS_TILE - 1) / BS_TILE;
        ring_entry& e = s->rh->ring[slot];
        e.d = r.d;
        e.tile_begin = s->rtiles;
        e.ntiles = ntiles;
        e.seq = seq;
        s->rtiles += ntiles;
        s->rseq = seq + 1;
        r.state = LAUNCHED;
        s->rpending.emplace_back(seq, r.id);
        any = true;
      }
      s->n_admitted.store((int)s->admitted.size(), std::memory_order_release);
      if (any) {
        __atomic_store_n(&s->rh->tail, s->rseq, __ATOMIC_RELEASE);
        s->st.batches++;
      }
      published = s->rseq;
      active = !s->rpending.empty() || !s->admitted.empty();
    }
    // the kernel: notice that it left; launch one while requests are not yet taken
    if (s->rrunning && cudaStreamQuery(s->rstream) != cudaErrorNotReady) {
      s->rrunning = false;
      const cudaError_t e = cudaStreamSynchronize(s->rstream);
      const uint32_t why = __atomic_load_n(&s->rh->status, __ATOMIC_ACQUIRE);
      if (e != cudaSuccess || why == RES_WAIT_TIMEOUT) {
        std::lock_guard<std::mutex> g(s->m);
        if (s->worker_error == NT2CUDA_OK)
          s->worker_error = e != cudaSuccess ? from_cuda(e, NT2CUDA_ERR_LAUNCH) : NT2CUDA_ERR_TIMEOUT;
      }
    }
    if (!s->rrunning && __atomic_load_n(&s->rh->consumed, __ATOMIC_ACQUIRE) < published) {
      s->rfirst = __atomic_load_n(&s->rh->consumed, __ATOMIC_ACQUIRE);
      __atomic_store_n(&s->rh->status, (uint32_t)RES_RUNNING, __ATOMIC_RELEASE);
      // the previous kernel left closing set and its tickets run ahead of the
      // published tiles (blocks that waited took tickets no tile got): clear
      // the one and bring the other back to the first tile not yet published
      cudaError_t e = cudaMemsetAsync(&s->rd->closing.v, 0, sizeof(uint64_t), s->rstream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(&s->rd->next.v, &s->rd->pub.v, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s->rstream);
      if (e == cudaSuccess) e = launch_resident(s);
      std::lock_guard<std::mutex> g(s->m);
      if (e != cudaSuccess) {
        if (s->worker_error == NT2CUDA_OK) s->worker_error = from_cuda(e, NT2CUDA_ERR_LAUNCH);
      } else {
        s->rrunning = true;
        s->st.launches++;
      }
    }
    // completions, in any order
    bool completed = false;
    {
      std::lock_guard<std::mutex> g(s->m);
      const uint64_t t = now_ns();
      for (auto it = s->rpending.begin(); it != s->rpending.end();) {
        const uint64_t seq = it->first;
        if (__atomic_load_n(&s->rh->done[seq % kRing], __ATOMIC_ACQUIRE) == seq + 1 || s->worker_error != NT2CUDA_OK) {
          auto q = s->reqs.find(it->second);
          if (q != s->reqs.end()) {
            q->second.state = DONE;
            q->second.t_done = t;
            s->st.completed++;
          }
          it = s->rpending.erase(it);
          completed = true;
        } else {
          ++it;
        }
      }
    }
    if (completed) s->cv_done.notify_all();
    if (active) {
      idle_since = now_ns();
      continue;                                     // poll while requests are outstanding
    }
    // idle: poll briefly for new requests, then sleep until one arrives
    if (now_ns() - idle_since < s->spin_ns) continue;
    std::unique_lock<std::mutex> lk(s->m);
    s->cv_work.wait_for(lk, std::chrono::milliseconds(2),
                        [&] { return s->stop || !s->admitted.empty() || !s->waiting.empty(); });
  }
  // stopping: let the kernel leave and wait for it
  __atomic_store_n(&s->rh->stop, 1u, __ATOMIC_RELEASE);
  if (s->rrunning) {
    cudaStreamSynchronize(s->rstream);
    s->rrunning = false;
  }
}

nt2cuda_status wait_done_locked(nt2cuda_server* s, std::unique_lock<std::mutex>& lk, uint64_t id, int timeout_ms)
{
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return NT2CUDA_ERR_ARG;
  if (it->second.state == DONE) return NT2CUDA_OK;
  if (timeout_ms == 0) return NT2CUDA_ERR_NOT_READY;
  auto pred = [&] {
    auto j = s->reqs.find(id);
    return j == s->reqs.end() || j->second.state == DONE;
  };
  if (timeout_ms < 0) timeout_ms = s->cfg.wait_timeout_ms;
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return NT2CUDA_ERR_TIMEOUT;
  return s->reqs.count(id) ? NT2CUDA_OK : NT2CUDA_ERR_ARG;
}

}  // namespace

extern "C" {

nt2cuda_status nt2cuda_server_create(const nt2cuda_server_config* cfg, nt2cuda_server** out)
{
  if (!cfg || !out) return NT2CUDA_ERR_ARG;
  *out = nullptr;
  if (cfg->budget_bytes < 4096 || cfg->max_inflight_batches < 1 || cfg->max_inflight_batches > 16 ||
      cfg->max_batch_requests < 1 || cfg->max_batch_requests > (1 << 20) || cfg->coalesce < 0 || cfg->coalesce > 2 ||
      (cfg->cdf_kind != CDF_NORMCDF && cfg->cdf_kind != CDF_FASTNORMCDF) || cfg->fused < 0 || cfg->fused > 2 ||
      cfg->spin_us > 100000)
    return NT2CUDA_ERR_ARG;
  nt2cuda_server* s = new nt2cuda_server();
  s->cfg = *cfg;
  if (s->cfg.wait_timeout_ms <= 0) s->cfg.wait_timeout_ms = 60000;
  s->spin_ns = cfg->spin_us < 0 ? 0 : (uint64_t)(cfg->spin_us == 0 ? 50 : cfg->spin_us) * 1000;
  cudaGetDevice(&s->device);
  if (!s->mem.init(cfg->budget_bytes)) { delete s; return NT2CUDA_ERR_OOM; }
  s->slots.resize((size_t)cfg->max_inflight_batches);
  const int maxb = cfg->coalesce ? cfg->max_batch_requests : 1;
  const size_t desc_bytes = ((size_t)maxb * sizeof(req_desc) + 255) / 256 * 256;
  const size_t slot_bytes = desc_bytes + ((size_t)maxb + 1) * 8;
  for (slot& sl : s->slots) {
    bool ok = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
              cudaMallocHost(&sl.h_buf, slot_bytes) == cudaSuccess &&
              cudaMalloc(&sl.d_buf, slot_bytes) == cudaSuccess;
    if (!ok) { nt2cuda_server_destroy(s); return NT2CUDA_ERR_OOM; }
    sl.bytes = slot_bytes;
    sl.h_desc = (req_desc*)sl.h_buf;
    sl.h_tiles = (uint64_t*)(sl.h_buf + desc_bytes);
    sl.d_desc = (req_desc*)sl.d_buf;
    sl.d_tiles = (uint64_t*)(sl.d_buf + desc_bytes);
  }
  if (s->cfg.coalesce == 2) {
    void* hp = nullptr;
    void* dp = nullptr;
    bool ok = cudaHostAlloc(&hp, sizeof(resident_host), cudaHostAllocMapped | cudaHostAllocPortable) == cudaSuccess;
    if (ok) {
      s->rh = (resident_host*)hp;
      std::memset(hp, 0, sizeof(resident_host));
      ok = cudaHostGetDevicePointer(&dp, hp, 0) == cudaSuccess;
      s->rh_dev = (resident_host*)dp;
    }
    ok = ok && cudaMalloc(&s->rd, sizeof(resident_dev)) == cudaSuccess &&
         cudaMemset(s->rd, 0, sizeof(resident_dev)) == cudaSuccess &&
         cudaStreamCreateWithFlags(&s->rstream, cudaStreamNonBlocking) == cudaSuccess &&
         cudaDeviceSynchronize() == cudaSuccess;
    if (!ok) { nt2cuda_server_destroy(s); return NT2CUDA_ERR_OOM; }
    s->rgrid = resident_grid(s->cfg);                  // also loads the kernel
    s->worker = std::thread(resident_loop, s);
    *out = s;
    return NT2CUDA_OK;
  }
  warm(s->cfg);
  s->worker = std::thread(worker_loop, s);
  s->reaper = std::thread(reaper_loop, s);
  *out = s;
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_server_destroy(nt2cuda_server* s)
{
  if (!s) return NT2CUDA_OK;
  {
    std::lock_guard<std::mutex> g(s->m);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  s->cv_inflight.notify_all();
  if (s->reaper.joinable()) s->reaper.join();   // drains every launched batch first
  for (slot& sl : s->slots) if (sl.stream) cudaStreamSynchronize(sl.stream);
  if (s->rstream) {
    cudaStreamSynchronize(s->rstream);
    cudaStreamDestroy(s->rstream);
  }
  if (s->rd) cudaFree(s->rd);
  if (s->rh) cudaFreeHost(s->rh);
  for (slot& sl : s->slots) {
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.h_buf) cudaFreeHost(sl.h_buf);
    if (sl.d_buf) cudaFree(sl.d_buf);
  }
  delete s;
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_server_submit(nt2cuda_server* s, const float* S, const float* K, const float* T, float r,
                                     float sigma, size_t n, uint64_t* ticket)
{
  if (!s || !ticket || n == 0 || !S || !K || !T) return NT2CUDA_ERR_ARG;
  const size_t half = (n * sizeof(float) + 255) / 256 * 256;
  const size_t bytes = 2 * half;
  if (bytes > s->cfg.budget_bytes) return NT2CUDA_ERR_BUDGET;
  {
    std::lock_guard<std::mutex> g(s->m);
    if (s->worker_error != NT2CUDA_OK) return s->worker_error;
    request q;
    q.id = s->next_id++;
    q.d.S = S;
    q.d.K = K;
    q.d.T = T;
    q.d.call = nullptr;
    q.d.put = nullptr;
    q.d.n = (uint64_t)n;
    q.d.r = r;
    q.d.sigma = sigma;
    // outputs are 256-aligned arena slots; inputs decide the vector path
    q.d.vec_ok = ((((uintptr_t)S | (uintptr_t)K | (uintptr_t)T) & 15u) == 0) ? 1u : 0u;
    q.d.pad = 0;
    q.bytes = bytes;
    q.t_submit = now_ns();
    s->reqs.emplace(q.id, q);
    s->waiting.push_back(q.id);
    s->st.submitted++;
    s->st.options += (uint64_t)n;
    size_t before = s->admitted.size();
    admit_locked(s);
    if (s->admitted.size() == before) s->st.admission_waits++;
    *ticket = q.id;
  }
  s->cv_work.notify_one();
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_server_poll(nt2cuda_server* s, uint64_t ticket, float** call, float** put)
{
  return nt2cuda_server_wait(s, ticket, 0, call, put);
}

nt2cuda_status nt2cuda_server_wait(nt2cuda_server* s, uint64_t ticket, int timeout_ms, float** call, float** put)
{
  if (!s) return NT2CUDA_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->m);
  nt2cuda_status st = wait_done_locked(s, lk, ticket, timeout_ms);
  if (st != NT2CUDA_OK) return st;
  const request& r = s->reqs[ticket];
  if (call) *call = r.d.call;
  if (put) *put = r.d.put;
  return s->worker_error;
}

nt2cuda_status nt2cuda_server_release(nt2cuda_server* s, uint64_t ticket)
{
  if (!s) return NT2CUDA_ERR_ARG;
  {
    std::lock_guard<std::mutex> g(s->m);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return NT2CUDA_ERR_ARG;
    if (it->second.state != DONE) return NT2CUDA_ERR_STATE;
    if (it->second.d.call) {
      s->mem.release(it->second.off, it->second.bytes);
      s->reserved -= it->second.bytes;
      s->st.reserved_bytes = s->reserved;
    }
    s->reqs.erase(it);
    admit_locked(s);
  }
  s->cv_work.notify_one();
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_server_latency_ns(nt2cuda_server* s, uint64_t ticket, uint64_t* ns)
{
  if (!s || !ns) return NT2CUDA_ERR_ARG;
  std::lock_guard<std::mutex> g(s->m);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return NT2CUDA_ERR_ARG;
  if (it->second.state != DONE) return NT2CUDA_ERR_NOT_READY;
  *ns = it->second.t_done - it->second.t_submit;
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_server_drain(nt2cuda_server* s, int timeout_ms)
{
  if (!s) return NT2CUDA_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->m);
  if (timeout_ms < 0) timeout_ms = s->cfg.wait_timeout_ms;
  auto pred = [&] {
    if (!s->waiting.empty() || !s->admitted.empty()) return false;
    for (auto& kv : s->reqs) if (kv.second.state != DONE) return false;
    return true;
  };
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return NT2CUDA_ERR_TIMEOUT;
  return s->worker_error;
}

nt2cuda_status nt2cuda_server_get_stats(nt2cuda_server* s, nt2cuda_server_stats* out)
{
  if (!s || !out) return NT2CUDA_ERR_ARG;
  std::lock_guard<std::mutex> g(s->m);
  *out = s->st;
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_server_replay(nt2cuda_server* s, const float* S, const float* K, const float* T, float r,
                                     float sigma, size_t nreq, const uint64_t* offsets, const uint64_t* sizes,
                                     const uint64_t* arrival_ns, uint64_t* latency_ns, uint64_t* elapsed_ns)
{
  if (!s || !S || !K || !T || (nreq && (!offsets || !sizes || !arrival_ns || !latency_ns)) || !elapsed_ns)
    return NT2CUDA_ERR_ARG;
  std::vector<uint64_t> tickets(nreq);
  std::atomic<size_t> submitted{0};
  std::atomic<int> err{NT2CUDA_OK};
  std::atomic<uint64_t> t_last{0};
  const uint64_t t0 = now_ns();
  std::thread collector([&] {
    for (size_t i = 0; i < nreq; ++i) {
      while (submitted.load(std::memory_order_acquire) <= i) {
        if (err.load(std::memory_order_acquire) != NT2CUDA_OK) return;
        std::this_thread::yield();
      }
      const uint64_t t = tickets[i];
      nt2cuda_status st = nt2cuda_server_wait(s, t, -1, nullptr, nullptr);
      if (st == NT2CUDA_OK) st = nt2cuda_server_latency_ns(s, t, &latency_ns[i]);
      if (st == NT2CUDA_OK) st = nt2cuda_server_release(s, t);
      if (st != NT2CUDA_OK) { int ok = NT2CUDA_OK; err.compare_exchange_strong(ok, (int)st); return; }
      t_last.store(now_ns(), std::memory_order_release);
    }
  });
  for (size_t i = 0; i < nreq && err.load(std::memory_order_acquire) == NT2CUDA_OK; ++i) {
    const uint64_t due = t0 + arrival_ns[i];
    while (now_ns() < due) {
    }
    uint64_t t = 0;
    nt2cuda_status st = nt2cuda_server_submit(s, S + offsets[i], K + offsets[i], T + offsets[i], r, sigma,
                                              (size_t)sizes[i], &t);
    if (st != NT2CUDA_OK) { int ok = NT2CUDA_OK; err.compare_exchange_strong(ok, (int)st); break; }
    tickets[i] = t;
    submitted.store(i + 1, std::memory_order_release);
  }
  collector.join();
  *elapsed_ns = t_last.load() > t0 ? t_last.load() - t0 : 0;
  return (nt2cuda_status)err.load();
}

}  // extern "C"
