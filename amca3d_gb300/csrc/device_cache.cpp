// device_cache.cpp — see device_cache.h.
#include "device_cache.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

namespace amca {
namespace {

struct DeviceCache {
  std::mutex m;
  std::vector<std::vector<std::pair<void *, size_t>>> slot;  // by device, largest first
};

// Never destroyed: the driver reclaims device memory at exit.
DeviceCache &cache() {
  static DeviceCache *c = new DeviceCache();
  return *c;
}

}  // namespace

void *cache_take(int device, size_t bytes, size_t *got) {
  bytes = std::max<size_t>(bytes, 1);
  DeviceCache &c = cache();
  {
    std::lock_guard<std::mutex> g(c.m);
    if (device >= 0 && (size_t)device < c.slot.size()) {
      auto &v = c.slot[(size_t)device];
      size_t best = v.size();
      for (size_t i = 0; i < v.size(); ++i)
        if (v[i].second >= bytes && v[i].second / 2 <= bytes && (best == v.size() || v[i].second < v[best].second))
          best = i;
      if (best < v.size()) {
        void *p = v[best].first;
        *got = v[best].second;
        v.erase(v.begin() + (long)best);
        return p;
      }
    }
  }
  void *p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  *got = bytes;
  return p;
}

void cache_give(int device, void *p, size_t bytes) {
  if (!p) return;
  DeviceCache &c = cache();
  std::vector<void *> drop;
  {
    std::lock_guard<std::mutex> g(c.m);
    if (device < 0) {
      drop.push_back(p);
    } else {
      if ((size_t)device >= c.slot.size()) c.slot.resize((size_t)device + 1);
      auto &v = c.slot[(size_t)device];
      v.emplace_back(p, bytes);
      std::sort(v.begin(), v.end(), [](const std::pair<void *, size_t> &a, const std::pair<void *, size_t> &b) {
        return a.second > b.second;
      });
      size_t total = 0, keep = 0;
      for (; keep < v.size() && total + v[keep].second <= kDeviceCacheBytes; ++keep) total += v[keep].second;
      for (size_t i = keep; i < v.size(); ++i) drop.push_back(v[i].first);
      v.resize(keep);
    }
  }
  for (void *q : drop) cudaFree(q);
}

bool cache_release(int device) {
  DeviceCache &c = cache();
  std::vector<void *> drop;
  {
    std::lock_guard<std::mutex> g(c.m);
    for (size_t d = 0; d < c.slot.size(); ++d)
      if (device < 0 || (size_t)device == d) {
        for (auto &a : c.slot[d]) drop.push_back(a.first);
        c.slot[d].clear();
      }
  }
  bool ok = true;
  for (void *p : drop) ok = cudaFree(p) == cudaSuccess && ok;
  return ok;
}

}  // namespace amca
