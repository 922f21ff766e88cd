// nt2cuda/tuning.cuh -- launch-parameter table filled by the autotuner.
//
// Each entry maps (kernel key, log2 size bucket) to the tuned parameters of
// that kernel: U, the groups a thread keeps in flight per grid-stride trip,
// and W, the grid size in waves of (SM count x resident blocks).  Lookups
// that miss return the defaults.  The table is process-wide and guarded by a
// mutex; tuning results are exported and imported as text so callers can
// persist them.
#pragma once
#include <mutex>
#include <map>
#include <string>
#include <sstream>
#include <stddef.h>

namespace nt2cuda {
namespace tuning {

struct params { int unroll = 2; int waves = 1; };

inline std::mutex& table_mutex() { static std::mutex m; return m; }
inline std::map<std::string, params>& table() { static std::map<std::string, params> t; return t; }

inline int size_bucket(size_t n)
{
  int b = 0;
  while (n > 1) { n >>= 1; ++b; }
  return b;
}

inline std::string make_key(const char* key, size_t n)
{
  std::string k(key ? key : "");
  k += "@";
  k += std::to_string(size_bucket(n));
  return k;
}

// The entry for (key, size bucket of n), or `def` when there is none.
inline params lookup(const char* key, size_t n, params def = params{})
{
  if (!key) return def;
  std::lock_guard<std::mutex> g(table_mutex());
  auto it = table().find(make_key(key, n));
  return it == table().end() ? def : it->second;
}

inline int unroll_for(const char* key, size_t n) { return lookup(key, n).unroll; }

inline void set(const char* key, size_t n, params p)
{
  std::lock_guard<std::mutex> g(table_mutex());
  table()[make_key(key, n)] = p;
}

// "key@bucket unroll waves" lines
inline std::string export_text()
{
  std::lock_guard<std::mutex> g(table_mutex());
  std::ostringstream os;
  for (auto& kv : table()) os << kv.first << " " << kv.second.unroll << " " << kv.second.waves << "\n";
  return os.str();
}

inline int import_text(const std::string& text)
{
  std::istringstream is(text);
  std::string key;
  int u, w, count = 0;
  std::lock_guard<std::mutex> g(table_mutex());
  while (is >> key >> u >> w) {
    if (u != 1 && u != 2 && u != 4) continue;
    if (w < 1 || w > 64) continue;
    table()[key] = params{u, w};
    ++count;
  }
  return count;
}

}  // namespace tuning
}  // namespace nt2cuda
