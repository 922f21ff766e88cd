// capi_core.cu -- device setup, table storage, streams, synthetic inputs and
// the tuning table of the nt2cuda C ABI.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <string>
#include "internal.cuh"
#include "nt2cuda/launch.cuh"
#include "nt2cuda/scratch.cuh"
#include "nt2cuda/tuning.cuh"

using namespace nt2cuda;
using namespace nt2cuda::detail_capi;

extern "C" {

const char* nt2cuda_status_string(int status)
{
  switch (status) {
    case NT2CUDA_OK: return "ok";
    case NT2CUDA_ERR_ARG: return "invalid argument";
    case NT2CUDA_ERR_OOM: return "out of memory";
    case NT2CUDA_ERR_BUDGET: return "request exceeds the device-memory budget";
    case NT2CUDA_ERR_LAUNCH: return "kernel launch failed";
    case NT2CUDA_ERR_TIMEOUT: return "bounded wait timed out";
    case NT2CUDA_ERR_CUDA: return "CUDA runtime error";
    case NT2CUDA_ERR_NOT_READY: return "not ready";
    case NT2CUDA_ERR_ALIAS: return "tables of one statement partially overlap";
    case NT2CUDA_ERR_STATE: return "object used in the wrong state";
    default: return "unknown status";
  }
}

int nt2cuda_version(void) { return 100; }

nt2cuda_status nt2cuda_init(int device)
{
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return from_cuda(e);
  if (device < 0 || device >= count) return NT2CUDA_ERR_ARG;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return from_cuda(e);
  e = cudaFree(nullptr);   // create the primary context now
  return from_cuda(e);
}

nt2cuda_status nt2cuda_device_info(int* sms, size_t* free_bytes, size_t* total_bytes)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return from_cuda(e);
  if (sms) {
    e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return from_cuda(e);
  }
  if (free_bytes || total_bytes) {
    size_t f = 0, t = 0;
    e = cudaMemGetInfo(&f, &t);
    if (e != cudaSuccess) return from_cuda(e);
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
  }
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_scratch_allocations(unsigned long long* count)
{
  if (!count) return NT2CUDA_ERR_ARG;
  nt2cuda::scratch_pool& P = nt2cuda::global_scratch_pool();
  std::lock_guard<std::mutex> g(P.m);
  *count = P.allocations;
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_last_cuda_error(int* code)
{
  if (!code) return NT2CUDA_ERR_ARG;
  *code = last_cuda_error();
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_alloc(size_t bytes, void** ptr)
{
  if (!ptr) return NT2CUDA_ERR_ARG;
  *ptr = nullptr;
  if (bytes == 0) return NT2CUDA_OK;
  return from_cuda(cudaMalloc(ptr, bytes), NT2CUDA_ERR_OOM);
}

nt2cuda_status nt2cuda_free(void* ptr) { return ptr ? from_cuda(cudaFree(ptr)) : NT2CUDA_OK; }

nt2cuda_status nt2cuda_alloc_host(size_t bytes, void** ptr)
{
  if (!ptr) return NT2CUDA_ERR_ARG;
  *ptr = nullptr;
  if (bytes == 0) return NT2CUDA_OK;
  return from_cuda(cudaMallocHost(ptr, bytes), NT2CUDA_ERR_OOM);
}

nt2cuda_status nt2cuda_free_host(void* ptr) { return ptr ? from_cuda(cudaFreeHost(ptr)) : NT2CUDA_OK; }

nt2cuda_status nt2cuda_memcpy_h2d(void* dst, const void* src, size_t bytes, nt2cuda_stream s)
{
  if (bytes && (!dst || !src)) return NT2CUDA_ERR_ARG;
  return from_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, as_stream(s)));
}

nt2cuda_status nt2cuda_memcpy_d2h(void* dst, const void* src, size_t bytes, nt2cuda_stream s)
{
  if (bytes && (!dst || !src)) return NT2CUDA_ERR_ARG;
  return from_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, as_stream(s)));
}

nt2cuda_status nt2cuda_memcpy_d2d(void* dst, const void* src, size_t bytes, nt2cuda_stream s)
{
  if (bytes && (!dst || !src)) return NT2CUDA_ERR_ARG;
  return from_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, as_stream(s)));
}

nt2cuda_status nt2cuda_stream_create(nt2cuda_stream* s)
{
  if (!s) return NT2CUDA_ERR_ARG;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  *s = reinterpret_cast<nt2cuda_stream>(st);
  return from_cuda(e);
}

nt2cuda_status nt2cuda_stream_destroy(nt2cuda_stream s)
{
  return s ? from_cuda(cudaStreamDestroy(as_stream(s))) : NT2CUDA_OK;
}

nt2cuda_status nt2cuda_stream_sync(nt2cuda_stream s) { return from_cuda(cudaStreamSynchronize(as_stream(s))); }

nt2cuda_status nt2cuda_tuning_export(char* buf, size_t cap, size_t* needed)
{
  std::string t = tuning::export_text();
  if (needed) *needed = t.size() + 1;
  if (!buf) return NT2CUDA_OK;
  if (cap < t.size() + 1) return NT2CUDA_ERR_ARG;
  memcpy(buf, t.c_str(), t.size() + 1);
  return NT2CUDA_OK;
}

nt2cuda_status nt2cuda_tuning_import(const char* text, int* entries)
{
  if (!text) return NT2CUDA_ERR_ARG;
  int n = tuning::import_text(std::string(text));
  if (entries) *entries = n;
  return NT2CUDA_OK;
}

}  // extern "C"

// ----------------------------------------------------------- generators
namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ uint64_t hash2(uint64_t seed, uint64_t i)
{
  return splitmix64(seed * 0xd1342543de82ef95ull + splitmix64(i));
}

// Uniform in [lo, hi): u = top 24 bits / 2^24 (exact in float), x = lo + (hi-lo)*u.
__global__ void k_fill_uniform_f32(float* x, size_t n, float lo, float hi, uint64_t seed)
{
  const float w = __fsub_rn(hi, lo);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float u = (float)(hash2(seed, i) >> 40) * (1.0f / 16777216.0f);
    x[i] = __fadd_rn(lo, __fmul_rn(w, u));
  }
}

__global__ void k_fill_uniform_f64(double* x, size_t n, double lo, double hi, uint64_t seed)
{
  const double w = __dsub_rn(hi, lo);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double u = (double)(hash2(seed, i) >> 11) * (1.0 / 9007199254740992.0);
    x[i] = __dadd_rn(lo, __dmul_rn(w, u));
  }
}

// N(0,1) by Box-Muller from two counter-based uniforms.
__global__ void k_fill_normal_f32(float* x, size_t n, uint64_t seed)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint64_t h = hash2(seed, i);
    float u1 = ((float)(h >> 40) + 1.0f) * (1.0f / 16777217.0f);
    float u2 = (float)((h >> 16) & 0xffffffull) * (1.0f / 16777216.0f);
    x[i] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
  }
}

template <class K, class... A>
nt2cuda_status launch_fill(K k, size_t n, cudaStream_t s, A... a)
{
  if (n == 0) return NT2CUDA_OK;
  size_t blocks = (n + 255) / 256;
  size_t cap = (size_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  k<<<(unsigned)blocks, 256, 0, s>>>(a...);
  return launch_status(cudaSuccess);
}

}  // namespace

extern "C" {

nt2cuda_status nt2cuda_fill_uniform_f32(float* x, size_t n, float lo, float hi, uint64_t seed, nt2cuda_stream s)
{
  if (n && !x) return NT2CUDA_ERR_ARG;
  return launch_fill(k_fill_uniform_f32, n, as_stream(s), x, n, lo, hi, seed);
}

nt2cuda_status nt2cuda_fill_uniform_f64(double* x, size_t n, double lo, double hi, uint64_t seed, nt2cuda_stream s)
{
  if (n && !x) return NT2CUDA_ERR_ARG;
  return launch_fill(k_fill_uniform_f64, n, as_stream(s), x, n, lo, hi, seed);
}

nt2cuda_status nt2cuda_fill_normal_f32(float* x, size_t n, uint64_t seed, nt2cuda_stream s)
{
  if (n && !x) return NT2CUDA_ERR_ARG;
  return launch_fill(k_fill_normal_f32, n, as_stream(s), x, n, seed);
}

}  // extern "C"
