// Fixed-point aggregation into caller-provided device buffers, with no device allocation.
//
// Who needs this: code that may not call cudaMalloc at the moment it wants the aggregation, for
// example a host that runs the library inside its own memory pool and forbids other allocations,
// code enqueueing work from a stream callback or between the launches of a latency-critical
// loop (cudaMalloc can synchronise the device), or an application that must keep its device
// footprint fixed after start-up. Such a caller hands in the fixed-point states it has and the
// buffers for the result; the only scratch is the hash table below, a file-scope device array
// that every GPU which loads libmbg.so holds until the process exits.
//
// Limits and sharing: at most kNoallocMaxStates states per call. All calls on one device share
// the one table; every call clears it on its own stream first, so calls queued on one stream are
// safe, but calls that overlap on the GPU (different streams, or different host threads without
// ordering) race on the table and give wrong counts.
#include <cuda.h>  // driver types only: the two driver calls below come through cudaGetDriverEntryPoint
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../../include/mbg.h"
#include "../host/devmem.hpp"

namespace mbg {
// Records the message for mbg_last_error() and returns `st` (defined with the C ABI, capi.cpp).
mbg_status set_error(mbg_status st, const std::string& msg);
}  // namespace mbg

namespace {

constexpr unsigned kNoallocSlots = 1u << 16;          // hash slots
constexpr unsigned kNoallocMaxStates = kNoallocSlots / 2;  // load factor at most 1/2
constexpr int kMaxDevices = 64;

// [0, slots): representative entry per slot, [slots, 2 slots): count per slot. 512 KiB.
static __device__ __align__(256) unsigned g_fp_scratch[2 * kNoallocSlots];

// The array's device address per device, with the id of the context it was looked up in: a new
// context on the device (after cudaDeviceReset the library's module is loaded again, possibly at
// another address) makes the next call look it up again.
struct ScratchAddr {
    unsigned long long ctx_id;  // 0: unknown, look the address up on every call
    unsigned* ptr;
};
std::mutex g_setup_mu;
ScratchAddr g_scratch_addr[kMaxDevices] = {};

__device__ __forceinline__ unsigned long long na_hash(const unsigned* w, int words) {
    unsigned long long h = 0x9E3779B97F4A7C15ull ^ (unsigned long long)words;
    for (int i = 0; i < words; ++i) {
        h ^= w[i];
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 29;
    }
    h *= 0x94D049BB133111EBull;
    return h ^ (h >> 32);
}

__device__ __forceinline__ bool na_same(const unsigned* a, const unsigned* b, int words) {
    for (int i = 0; i < words; ++i)
        if (a[i] != b[i]) return false;
    return true;
}

// Same insertion as mbg_fp_insert, with the entry count passed by value and the table in the
// static scratch array. The table has twice as many slots as entries, so a probe always ends.
__global__ void fp_insert_noalloc(const unsigned* __restrict__ states, unsigned n, int words,
                                  unsigned* __restrict__ scratch) {
    unsigned* rep = scratch;
    unsigned* cnt = scratch + kNoallocSlots;
    const unsigned mask = kNoallocSlots - 1u;
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const unsigned* me = states + (unsigned long long)e * words;
        unsigned s = (unsigned)na_hash(me, words) & mask;
        for (unsigned probe = 0; probe <= mask; ++probe) {
            unsigned cur = atomicCAS(rep + s, 0xFFFFFFFFu, e);
            if (cur == 0xFFFFFFFFu || na_same(states + (unsigned long long)cur * words, me, words)) {
                atomicAdd(cnt + s, 1u);
                break;
            }
            s = (s + 1u) & mask;
        }
    }
}

__global__ void fp_compact_noalloc(const unsigned* __restrict__ states, int words, const unsigned* __restrict__ scratch,
                                   unsigned* __restrict__ out_states, unsigned* __restrict__ out_cnt,
                                   unsigned* __restrict__ n_unique) {
    const unsigned* rep = scratch;
    const unsigned* cnt = scratch + kNoallocSlots;
    for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < kNoallocSlots; s += gridDim.x * blockDim.x) {
        unsigned r = rep[s];
        if (r != 0xFFFFFFFFu) {
            unsigned o = atomicAdd(n_unique, 1u);
            out_cnt[o] = cnt[s];
            for (int w = 0; w < words; ++w)
                out_states[(unsigned long long)o * words + w] = states[(unsigned long long)r * words + w];
        }
    }
}

// Device address of the scratch array on the current device: looked up with the device current,
// once per device and context (the first call on a device, and the first after its context was
// replaced, does the lookup).
cudaError_t scratch_for_current_device(unsigned** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    unsigned long long id = 0;
    bool have_id = mbg::current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    ScratchAddr& a = g_scratch_addr[dev];
    if (have_id && a.ptr && a.ctx_id == id) {
        *out = a.ptr;
        return cudaSuccess;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_fp_scratch);  // also creates the context if it did not exist yet
    if (e != cudaSuccess) return e;
    if (!have_id) have_id = mbg::current_context_id(&id);
    a.ptr = static_cast<unsigned*>(p);
    a.ctx_id = have_id ? id : 0ull;
    *out = a.ptr;
    return cudaSuccess;
}

}  // namespace

extern "C" mbg_status mbg_fixed_points_aggregate_noalloc(const uint32_t* states, uint32_t n_states, int32_t words,
                                                         uint32_t* unique_states, uint32_t* counts,
                                                         uint32_t* n_unique, void* stream) {
    if (n_states > kNoallocMaxStates)
        return mbg::set_error(MBG_ERR_ARG, "mbg_fixed_points_aggregate_noalloc: " + std::to_string(n_states) +
                                               " states exceed the limit of " + std::to_string(kNoallocMaxStates) +
                                               " per call");
    if (words < 1 || !n_unique || (n_states > 0 && (!states || !unique_states || !counts)))
        return mbg::set_error(MBG_ERR_ARG, "mbg_fixed_points_aggregate_noalloc: null buffer or words < 1");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Every status below is the return value of its own call: an error the caller left pending
    // in the runtime's error state is neither cleared nor reported as this call's.
    unsigned* scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0xFF, sizeof(unsigned) * kNoallocSlots, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + kNoallocSlots, 0, sizeof(unsigned) * kNoallocSlots, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(n_unique, 0, sizeof(unsigned), st);
    if (e == cudaSuccess && n_states > 0) {
        void* ins[] = {(void*)&states, (void*)&n_states, (void*)&words, (void*)&scratch};
        e = cudaLaunchKernel((const void*)fp_insert_noalloc, dim3(128), dim3(256), ins, 0, st);
        if (e == cudaSuccess) {
            void* cmp[] = {(void*)&states, (void*)&words, (void*)&scratch, (void*)&unique_states, (void*)&counts,
                           (void*)&n_unique};
            e = cudaLaunchKernel((const void*)fp_compact_noalloc, dim3(128), dim3(256), cmp, 0, st);
        }
    }
    if (e != cudaSuccess)
        return mbg::set_error(MBG_ERR_CUDA, std::string("mbg_fixed_points_aggregate_noalloc: ") + cudaGetErrorString(e));
    return mbg::set_error(MBG_OK, "");
}
