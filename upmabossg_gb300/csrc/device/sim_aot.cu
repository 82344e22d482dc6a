// Kernels compiled ahead of time for sm_103a: the warp-per-trajectory simulator and the
// fixed-point aggregation. The thread-per-trajectory simulator is compiled per model by NVRTC
// from the same headers (see jit.cpp).
#include <cuda_runtime.h>

#include "philox.h"
#include "sim_types.h"
#include "sim_core.cuh"
#include "sim_warp.cuh"
#include "kernels.h"

namespace mbg {

extern "C" __global__ void __launch_bounds__(256) mbg_sim_warp(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_warp_body(p, smem);
}

// ---------------------------------------------------------------------------------------------
// Fixed points (src/statistics/fixed_states.cu:84-125 selects, sorts and run-length encodes the
// fixed states of every batch, then merges them into a host map). Here every fixed-point
// trajectory appended its state to `fp_states` during the simulation; one pass inserts each
// entry into an open-addressing table whose slots hold the index of a representative entry.
// All entries exist before this kernel starts, so a probe only compares immutable states and
// never waits on another thread.

__device__ __forceinline__ unsigned long long hash_words(const unsigned* w, int words) {
    unsigned long long h = 0x9E3779B97F4A7C15ull ^ (unsigned long long)words;
    for (int i = 0; i < words; ++i) {
        h ^= w[i];
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 29;
    }
    h *= 0x94D049BB133111EBull;
    return h ^ (h >> 32);
}

__device__ __forceinline__ bool same_words(const unsigned* a, const unsigned* b, int words) {
    for (int i = 0; i < words; ++i)
        if (a[i] != b[i]) return false;
    return true;
}

extern "C" __global__ void mbg_fp_insert(const unsigned* __restrict__ fp_states, const unsigned* __restrict__ fp_count,
                                         unsigned capacity, int words, unsigned* __restrict__ slot_rep,
                                         unsigned* __restrict__ slot_cnt, unsigned mask,
                                         unsigned* __restrict__ error_flag) {
    unsigned n = *fp_count;
    if (n > capacity) n = capacity;
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const unsigned* me = fp_states + (unsigned long long)e * words;
        unsigned s = (unsigned)hash_words(me, words) & mask;
        bool placed = false;
        for (unsigned probe = 0; probe <= mask; ++probe) {
            unsigned cur = atomicCAS(slot_rep + s, 0xFFFFFFFFu, e);
            if (cur == 0xFFFFFFFFu || same_words(fp_states + (unsigned long long)cur * words, me, words)) {
                atomicAdd(slot_cnt + s, 1u);
                placed = true;
                break;
            }
            s = (s + 1u) & mask;
        }
        if (!placed) atomicOr(error_flag, (unsigned)DEV_ERR_FP_OVERFLOW);
    }
}

extern "C" __global__ void mbg_fp_compact(const unsigned* __restrict__ fp_states, int words,
                                          const unsigned* __restrict__ slot_rep, const unsigned* __restrict__ slot_cnt,
                                          unsigned n_slots, unsigned* __restrict__ out_states,
                                          unsigned* __restrict__ out_cnt, unsigned* __restrict__ n_unique) {
    for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n_slots; s += gridDim.x * blockDim.x) {
        unsigned r = slot_rep[s];
        if (r != 0xFFFFFFFFu) {
            unsigned o = atomicAdd(n_unique, 1u);
            out_cnt[o] = slot_cnt[s];
            for (int w = 0; w < words; ++w)
                out_states[(unsigned long long)o * words + w] = fp_states[(unsigned long long)r * words + w];
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Host-side launchers.

cudaError_t launch_sim_warp(const SimParams& p, int grid, int block, size_t smem, cudaStream_t stream) {
    mbg_sim_warp<<<grid, block, smem, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t sim_warp_configure(size_t smem) {
    return cudaFuncSetAttribute(mbg_sim_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

unsigned sim_warp_smem_per_warp(int n) { return warp_smem_bytes(n); }

cudaError_t sim_warp_occupancy(int block, size_t smem, int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, mbg_sim_warp, block, smem);
}

cudaError_t launch_fp_aggregate(const unsigned* fp_states, const unsigned* fp_count, unsigned capacity, int words,
                                unsigned* slot_rep, unsigned* slot_cnt, unsigned n_slots, unsigned* out_states,
                                unsigned* out_cnt, unsigned* n_unique, unsigned* error_flag, int sms,
                                cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(slot_rep, 0xFF, sizeof(unsigned) * n_slots, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(slot_cnt, 0, sizeof(unsigned) * n_slots, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(n_unique, 0, sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    mbg_fp_insert<<<sms * 4, 256, 0, stream>>>(fp_states, fp_count, capacity, words, slot_rep, slot_cnt,
                                               n_slots - 1u, error_flag);
    mbg_fp_compact<<<sms * 4, 256, 0, stream>>>(fp_states, words, slot_rep, slot_cnt, n_slots, out_states, out_cnt,
                                                n_unique);
    return cudaGetLastError();
}

}  // namespace mbg
