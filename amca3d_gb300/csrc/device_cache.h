// device_cache.h — device allocations kept for reuse after a realm is destroyed.
//
// A realm's device buffers (the plain realm's one arena, the remelting
// realm's per-array buffers) go back here when its handle is destroyed (once
// its stream is idle) and are reused by the realms created after it on the
// same device: the next deck of a sweep, the next end-to-end run, the next
// batch of instances. Up to kDeviceCacheBytes per device are kept, larger
// buffers first. Every buffer is initialized (or written before it is read)
// by its new owner, as after a fresh cudaMalloc.
#pragma once

#include <stddef.h>

namespace amca {

constexpr size_t kDeviceCacheBytes = 32ull << 30;

// A buffer of at least `bytes` on `device` (the current device): the smallest
// kept one that fits without wasting more than half of it, else cudaMalloc.
// *got = its size. Returns nullptr when cudaMalloc fails.
void *cache_take(int device, size_t bytes, size_t *got);

// Back to the cache (or cudaFree when the cache is full of larger buffers).
void cache_give(int device, void *p, size_t bytes);

// cudaFree every kept buffer of `device` (every device when device < 0);
// false when a cudaFree failed.
bool cache_release(int device);

}  // namespace amca
