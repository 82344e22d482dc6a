// Device and pinned host blocks of the simulation handles, through a process-wide cache.
//
// A freed block is kept, keyed by its context and size, and handed to the next allocation of that
// size in that context: creating and destroying handles of one shape (a sweep driver, repeated
// runs of one model in a process) then costs no cudaMalloc or cudaFree, and no implicit device
// synchronisation, after the first. At most kDevCacheBytes of device blocks and kPinnedCacheBytes
// of pinned host blocks are kept; a block freed beyond that is released. Contexts are told apart
// by their unique id, so a block of a context that no longer exists (cudaDeviceReset) is never
// handed out again; without a context id nothing is cached, nor with MBG_DEVICE_CACHE=0 in the
// environment.
#pragma once

#include <cstddef>

namespace mbg {

constexpr size_t kDevCacheBytes = 16ull << 30;
constexpr size_t kPinnedCacheBytes = 64ull << 20;

// Unique id of the current context (cuCtxGetCurrent + cuCtxGetId through the runtime's driver entry
// points, so the library needs no link against libcuda); false if there is none or no entry point.
bool current_context_id(unsigned long long* id);

// Device block of `bytes` (at least 1) on the current device; throws NoMemError naming `what`.
void* dev_alloc(size_t bytes, const char* what);
// Returns a dev_alloc block (null: nothing). The caller guarantees that no pending work reads or
// writes it.
void dev_free(void* p);
// The same for page-locked host blocks.
void* pinned_alloc(size_t bytes);
void pinned_free(void* p);

}  // namespace mbg
