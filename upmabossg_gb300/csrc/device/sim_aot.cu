// Kernels compiled ahead of time for sm_103a: the warp-per-trajectory simulator and the
// fixed-point aggregation. The thread-per-trajectory simulator is compiled per model by NVRTC
// from the same headers (see jit.cpp).
#include <cuda_runtime.h>

#include <cmath>

#include "philox.h"
#include "sim_types.h"
#include "sim_core.cuh"
#include "sim_warp.cuh"
#include "sim_lane.cuh"
#include "kernels.h"

#include <utility>

namespace mbg {

// Cached-index variant (regulator index of every node kept in shared memory).
extern "C" __global__ void __launch_bounds__(256, 4) mbg_sim_warp(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_warp_body<true>(p, smem);
}

// Gather variant, for models whose index cache would not fit beside enough warps.
extern "C" __global__ void __launch_bounds__(256, 4) mbg_sim_warp_gather(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_warp_body<false>(p, smem);
}

// One trajectory per lane, state in shared memory, incremental rates; the readers of a flipped
// node are updated by their own lane, or dealt out over the warp (cooperative variant). The
// `_full` kernels also handle multi-valued (palette) rates and nodes over more than 12
// regulators; the others leave those paths out (a smaller loop body, 11-18% faster). Shared
// memory, not registers, bounds their residency where they are fastest (512 trajectories per SM
// at 1000 nodes), so they may use up to 128 registers: at 106 instead of 80 the 1000-node
// workload runs 4% faster (6.95e9 against 6.66e9 transitions/s).
extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, false>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_coop(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<true, false>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_full(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, true>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_coop_full(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<true, true>(p, smem);
}

// The lane layout with each block's rows in global memory instead of shared memory, for networks
// whose rows leave too few trajectories resident in shared memory: occupancy is then bounded by
// registers (three blocks of 256), the rows are cached in L1 (the whole carve-out) and L2. Per-lane
// reader update only (the cooperative one patches other lanes' rows with atomics).
extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_global(const SimParams p) {
    sim_lane_body<false, false>(p, p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_global_full(const SimParams p) {
    sim_lane_body<false, true>(p, p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes);
}

// The lane layout with the Fenwick tree and the state rows in shared memory and the active-word
// rows (read once per re-evaluated reader and once per walked group) in global memory, per block
// as in the global-row kernels: 256 instead of 384 bytes of shared memory per trajectory at 1000
// nodes, so three resident blocks of 256 per SM instead of two, at 80 registers (per-lane reader
// update).
extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_split(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, false>(p, smem,
                                reinterpret_cast<unsigned*>(p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes));
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_split_full(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, true>(p, smem,
                               reinterpret_cast<unsigned*>(p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes));
}

// Batched instances (parameter sweeps) in the lane layout, both reader-update variants.
extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_batch_body<false, false>(b, smem);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_coop(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_batch_body<true, false>(b, smem);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_full(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_batch_body<false, true>(b, smem);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_coop_full(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_batch_body<true, true>(b, smem);
}

// Batched instances in the lane layout with the active-word rows in global memory (per-lane reader
// update), as mbg_sim_lane_split: for size classes whose shared-memory rows hold fewer than three
// blocks of 256 per SM.
extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_split(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_batch_body<false, false>(b, smem,
                                      reinterpret_cast<unsigned*>(b.lane_state + (size_t)blockIdx.x * b.lane_block_bytes));
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_split_full(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_batch_body<false, true>(b, smem,
                                     reinterpret_cast<unsigned*>(b.lane_state + (size_t)blockIdx.x * b.lane_block_bytes));
}

// Batched instances in the lane layout with each block's rows in global memory (per-lane reader
// update): for size classes whose rows leave few trajectories resident in shared memory.
extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_global(const BatchDesc b) {
    sim_lane_batch_body<false, false>(b, b.lane_state + (size_t)blockIdx.x * b.lane_block_bytes);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_batch_global_full(const BatchDesc b) {
    sim_lane_batch_body<false, true>(b, b.lane_state + (size_t)blockIdx.x * b.lane_block_bytes);
}

// Batched instances (parameter sweeps) in the warp layout, both variants.
extern "C" __global__ void __launch_bounds__(256, 4) mbg_sim_warp_batch(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_warp_batch_body<true>(b, smem);
}

extern "C" __global__ void __launch_bounds__(256) mbg_sim_warp_batch_gather(const BatchDesc b) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_warp_batch_body<false>(b, smem);
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

// Batched aggregation: blockIdx.y selects the instance.
extern "C" __global__ void mbg_fp_insert_batch(const SimParams* __restrict__ params, const FpSlots* __restrict__ fps) {
    const SimParams& p = params[blockIdx.y];
    const FpSlots f = fps[blockIdx.y];
    unsigned n = *p.fp_count;
    if (n > p.fp_capacity) n = p.fp_capacity;
    const int words = p.words;
    const unsigned mask = f.n_slots - 1u;
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const unsigned* me = p.fp_states + (unsigned long long)e * words;
        unsigned s = (unsigned)hash_words(me, words) & mask;
        bool placed = false;
        for (unsigned probe = 0; probe <= mask; ++probe) {
            const unsigned cur = atomicCAS(f.slot_rep + s, 0xFFFFFFFFu, e);
            if (cur == 0xFFFFFFFFu || same_words(p.fp_states + (unsigned long long)cur * words, me, words)) {
                atomicAdd(f.slot_cnt + s, 1u);
                placed = true;
                break;
            }
            s = (s + 1u) & mask;
        }
        if (!placed) atomicOr(p.error_flag, (unsigned)DEV_ERR_FP_OVERFLOW);
    }
}

extern "C" __global__ void mbg_fp_compact_batch(const SimParams* __restrict__ params, const FpSlots* __restrict__ fps) {
    const SimParams& p = params[blockIdx.y];
    const FpSlots f = fps[blockIdx.y];
    const int words = p.words;
    for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < f.n_slots; s += gridDim.x * blockDim.x) {
        const unsigned r = f.slot_rep[s];
        if (r != 0xFFFFFFFFu) {
            const unsigned o = atomicAdd(f.n_unique, 1u);
            f.out_cnt[o] = f.slot_cnt[s];
            for (int w = 0; w < words; ++w)
                f.out_states[(unsigned long long)o * words + w] = p.fp_states[(unsigned long long)r * words + w];
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Host-side launchers. Each returns the status of its own launches (cudaLaunchKernelEx), so that
// an error the caller left pending in the runtime's error state is neither cleared nor reported
// as this library's.

namespace {
template <class K, class... A>
cudaError_t launch(K kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t stream, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}
}  // namespace

cudaError_t launch_sim_warp_batch(const BatchDesc& b, bool cached_index, int grid, int block, size_t smem,
                                  cudaStream_t stream) {
    return launch(cached_index ? mbg_sim_warp_batch : mbg_sim_warp_batch_gather, grid, block, smem, stream, b);
}

cudaError_t sim_warp_batch_configure(bool cached_index, size_t smem, int block, int* blocks_per_sm) {
    const void* f = cached_index ? (const void*)mbg_sim_warp_batch : (const void*)mbg_sim_warp_batch_gather;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, smem);
}

unsigned sim_warp_batch_slice_bytes(int max_n, bool cached_index) {
    return batch_params_bytes() + ((warp_smem_bytes(max_n, cached_index) + 15u) & ~15u);
}

cudaError_t launch_fp_aggregate_batch(const SimParams* params, const FpSlots* fps, int n_inst, int blocks_x,
                                      cudaStream_t stream) {
    dim3 grid(blocks_x, n_inst);
    cudaError_t e = launch(mbg_fp_insert_batch, grid, 256, 0, stream, params, fps);
    if (e != cudaSuccess) return e;
    return launch(mbg_fp_compact_batch, grid, 256, 0, stream, params, fps);
}

cudaError_t launch_sim_warp(const SimParams& p, bool cached_index, int grid, int block, size_t smem,
                            cudaStream_t stream) {
    if (p.hash_bits > 0) return cudaErrorInvalidValue;  // the warp layout runs on the dense window table only
    return launch(cached_index ? mbg_sim_warp : mbg_sim_warp_gather, grid, block, smem, stream, p);
}

cudaError_t sim_warp_configure(bool cached_index, size_t smem) {
    return cached_index ? cudaFuncSetAttribute(mbg_sim_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                        : cudaFuncSetAttribute(mbg_sim_warp_gather, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
}

unsigned sim_warp_smem_per_warp(int n, bool cached_index) { return warp_smem_bytes(n, cached_index); }

cudaError_t sim_warp_occupancy(bool cached_index, int block, size_t smem, int* blocks_per_sm) {
    return cached_index ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, mbg_sim_warp, block, smem)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, mbg_sim_warp_gather, block,
                                                                        smem);
}

cudaError_t launch_sim_lane(const SimParams& p, bool coop, bool full, int grid, int block, size_t smem,
                            cudaStream_t stream) {
    if (p.hash_bits > 0)
        return launch((void (*)(SimParams))sim_kernel_hash(full ? 4 : 0, coop), grid, block, smem, stream, p);
    auto k = full ? (coop ? mbg_sim_lane_coop_full : mbg_sim_lane_full) : (coop ? mbg_sim_lane_coop : mbg_sim_lane);
    return launch(k, grid, block, smem, stream, p);
}

namespace {

// Occupancy of a lane-layout kernel with the smallest shared-memory carve-out that keeps as many
// blocks resident: the rest of the SM's 256 KiB is L1, which caches the model tables every step
// reads. The driver rounds the percentage up to a supported carve-out, so the largest percentage
// at or below the need is tried first, then larger ones if that carve-out holds fewer blocks.
cudaError_t lane_configure(const void* f, size_t smem, int block, int* blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, smem);
    if (e != cudaSuccess || *blocks_per_sm < 1) return e;
    int dev = 0, per_sm = 0, reserved = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (e != cudaSuccess || per_sm <= 0) return e;
    const int want = *blocks_per_sm;
    const double need = (double)want * (double)(smem + (size_t)reserved);
    const int lo = (int)std::floor(100.0 * need / per_sm), hi = (int)std::ceil(100.0 * need / per_sm);
    for (int pct : {lo, hi, 100}) {
        e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct < 100 ? pct : 100);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, smem);
        if (e != cudaSuccess || *blocks_per_sm >= want) return e;
    }
    return e;
}

// Attributes of one kernel shared by several launch shapes (blocks[i], smems[i], want[i] resident
// blocks per SM): the largest dynamic shared memory of any shape and the smallest carve-out at
// which every shape keeps its resident blocks.
cudaError_t shared_limits(const void* f, const int* blocks, const size_t* smems, const int* want, int count) {
    size_t max_smem = 0;
    double need = 0;
    int dev = 0, per_sm = 0, reserved = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (e != cudaSuccess || per_sm <= 0) return e;
    for (int i = 0; i < count; ++i) {
        max_smem = smems[i] > max_smem ? smems[i] : max_smem;
        const double d = (double)want[i] * (double)(smems[i] + (size_t)reserved);
        need = d > need ? d : need;
    }
    e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
    if (e != cudaSuccess) return e;
    const int lo = (int)std::floor(100.0 * need / per_sm), hi = (int)std::ceil(100.0 * need / per_sm);
    for (int pct : {lo, hi, 100}) {
        e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct < 100 ? pct : 100);
        if (e != cudaSuccess) return e;
        bool ok = true;
        for (int i = 0; i < count && ok; ++i) {
            int bps = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, f, blocks[i], smems[i]);
            if (e != cudaSuccess) return e;
            ok = bps >= want[i];
        }
        if (ok) return cudaSuccess;
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t sim_kernel_limits(int kernel, bool variant, const int* blocks, const size_t* smems, const int* want,
                              int count, bool hash) {
    const void* f = hash ? sim_kernel_hash(kernel, variant) : nullptr;
    if (hash && !f) return cudaErrorInvalidValue;
    if (!f) switch (kernel) {
        case 0: f = variant ? (const void*)mbg_sim_lane_coop : (const void*)mbg_sim_lane; break;
        case 1: f = variant ? (const void*)mbg_sim_lane_batch_coop : (const void*)mbg_sim_lane_batch; break;
        case 4: f = variant ? (const void*)mbg_sim_lane_coop_full : (const void*)mbg_sim_lane_full; break;
        case 5: f = variant ? (const void*)mbg_sim_lane_batch_coop_full : (const void*)mbg_sim_lane_batch_full; break;
        case 2: f = variant ? (const void*)mbg_sim_warp_batch : (const void*)mbg_sim_warp_batch_gather; break;
        case 6: f = variant ? (const void*)mbg_sim_lane_global_full : (const void*)mbg_sim_lane_global; break;
        case 7: f = variant ? (const void*)mbg_sim_lane_batch_global_full : (const void*)mbg_sim_lane_batch_global; break;
        case 8: f = variant ? (const void*)mbg_sim_lane_split_full : (const void*)mbg_sim_lane_split; break;
        case 9: f = variant ? (const void*)mbg_sim_lane_batch_split_full : (const void*)mbg_sim_lane_batch_split; break;
        default: f = variant ? (const void*)mbg_sim_warp : (const void*)mbg_sim_warp_gather; break;
    }
    return shared_limits(f, blocks, smems, want, count);
}

cudaError_t sim_lane_configure(bool coop, bool full, size_t smem, int block, int* blocks_per_sm) {
    const void* f = full ? (coop ? (const void*)mbg_sim_lane_coop_full : (const void*)mbg_sim_lane_full)
                         : (coop ? (const void*)mbg_sim_lane_coop : (const void*)mbg_sim_lane);
    return lane_configure(f, smem, block, blocks_per_sm);
}

cudaError_t launch_sim_lane_batch(const BatchDesc& b, bool coop, bool full, int grid, int block, size_t smem,
                                  cudaStream_t stream) {
    auto k = full ? (coop ? mbg_sim_lane_batch_coop_full : mbg_sim_lane_batch_full)
                  : (coop ? mbg_sim_lane_batch_coop : mbg_sim_lane_batch);
    return launch(k, grid, block, smem, stream, b);
}

cudaError_t sim_lane_batch_configure(bool coop, bool full, size_t smem, int block, int* blocks_per_sm) {
    const void* f = full ? (coop ? (const void*)mbg_sim_lane_batch_coop_full : (const void*)mbg_sim_lane_batch_full)
                         : (coop ? (const void*)mbg_sim_lane_batch_coop : (const void*)mbg_sim_lane_batch);
    return lane_configure(f, smem, block, blocks_per_sm);
}

size_t sim_lane_smem(int n, int block) { return (size_t)block * lane_smem_bytes(n); }

cudaError_t sim_lane_batch_global_configure(bool full, int block, int* blocks_per_sm) {
    const void* f = full ? (const void*)mbg_sim_lane_batch_global_full : (const void*)mbg_sim_lane_batch_global;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 0);  // all L1
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, 0);
}

cudaError_t launch_sim_lane_batch_global(const BatchDesc& b, bool full, int grid, int block, cudaStream_t stream) {
    return launch(full ? mbg_sim_lane_batch_global_full : mbg_sim_lane_batch_global, grid, block, 0, stream, b);
}

cudaError_t sim_lane_global_configure(bool full, int block, int* blocks_per_sm) {
    const void* f = full ? (const void*)mbg_sim_lane_global_full : (const void*)mbg_sim_lane_global;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 0);  // all L1
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, 0);
}

cudaError_t launch_sim_lane_global(const SimParams& p, bool full, int grid, int block, cudaStream_t stream) {
    if (p.hash_bits > 0)
        return launch((void (*)(SimParams))sim_kernel_hash(6, full), grid, block, 0, stream, p);
    return launch(full ? mbg_sim_lane_global_full : mbg_sim_lane_global, grid, block, 0, stream, p);
}

int sim_lane_rows(int n) { return lane_groups(n); }

size_t sim_lane_split_smem(int n, int block) {
    const int G = lane_groups(n);
    return (size_t)block * (8u * (unsigned)lane_leaves(G, lane_leaf_shift(G)) + 4u * (unsigned)G);
}

cudaError_t sim_lane_batch_split_configure(bool full, size_t smem, int block, int* blocks_per_sm) {
    return lane_configure(full ? (const void*)mbg_sim_lane_batch_split_full : (const void*)mbg_sim_lane_batch_split,
                          smem, block, blocks_per_sm);
}

cudaError_t launch_sim_lane_batch_split(const BatchDesc& b, bool full, int grid, int block, size_t smem,
                                        cudaStream_t stream) {
    return launch(full ? mbg_sim_lane_batch_split_full : mbg_sim_lane_batch_split, grid, block, smem, stream, b);
}

cudaError_t sim_lane_split_configure(bool full, size_t smem, int block, int* blocks_per_sm) {
    return lane_configure(full ? (const void*)mbg_sim_lane_split_full : (const void*)mbg_sim_lane_split, smem, block,
                          blocks_per_sm);
}

cudaError_t launch_sim_lane_split(const SimParams& p, bool full, int grid, int block, size_t smem,
                                  cudaStream_t stream) {
    if (p.hash_bits > 0)
        return launch((void (*)(SimParams))sim_kernel_hash(8, full), grid, block, smem, stream, p);
    return launch(full ? mbg_sim_lane_split_full : mbg_sim_lane_split, grid, block, smem, stream, p);
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
    e = launch(mbg_fp_insert, sms * 4, 256, 0, stream, fp_states, fp_count, capacity, words, slot_rep, slot_cnt,
               n_slots - 1u, error_flag);
    if (e != cudaSuccess) return e;
    return launch(mbg_fp_compact, sms * 4, 256, 0, stream, fp_states, words, slot_rep, slot_cnt, n_slots, out_states,
                  out_cnt, n_unique);
}

}  // namespace mbg
