// nt2cuda/wait_status.cuh -- host-side registry of the device counters that
// record bounded waits which ran out.
//
// Kernels that wait on other blocks of their grid (the scan look-back) or on
// their own bulk copies (the TMA folds) count every wait that gives up in a
// `static __device__` counter of their translation unit.  Each translation
// unit is a module of its own, so a counter cannot be shared between them;
// instead every unit registers a host function that reads its counter, and
// nt2cuda_wait_timeouts adds them all up.
#pragma once
#include <cuda_runtime.h>
#include <mutex>
#include <vector>

namespace nt2cuda {

using timeout_reader = cudaError_t (*)(unsigned long long*);

struct timeout_registry {
  std::mutex m;
  std::vector<timeout_reader> readers;
};
inline timeout_registry& timeout_readers()
{
  static timeout_registry r;
  return r;
}

struct timeout_reader_registration {
  explicit timeout_reader_registration(timeout_reader f)
  {
    timeout_registry& r = timeout_readers();
    std::lock_guard<std::mutex> g(r.m);
    for (timeout_reader x : r.readers)
      if (x == f) return;
    r.readers.push_back(f);
  }
};

// Sum of every registered counter (synchronous: each read is a device-to-host copy).
inline cudaError_t total_wait_timeouts(unsigned long long* count)
{
  timeout_registry& r = timeout_readers();
  std::lock_guard<std::mutex> g(r.m);
  unsigned long long sum = 0;
  for (timeout_reader f : r.readers) {
    unsigned long long c = 0;
    cudaError_t e = f(&c);
    if (e != cudaSuccess) return e;
    sum += c;
  }
  *count = sum;
  return cudaSuccess;
}

}  // namespace nt2cuda
