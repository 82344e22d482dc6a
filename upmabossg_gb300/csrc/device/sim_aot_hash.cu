// The lane-layout single-simulation kernels of sim_aot.cu compiled with their window sums going to
// the window hash table (MBG_WINDOW_HASH, sim_core.cuh:bin_add) instead of the dense table. Same
// layouts, same arithmetic; launched when a run's table is the hash table (large, sparse output
// spaces). The warp layout has no such twin: on the GB300 its hash form stalled or mis-picked
// whenever the table overflowed, so the warp layout keeps the dense table (see sim.cpp).
#define MBG_WINDOW_HASH 1

#include <cuda_runtime.h>

#include <cmath>
#include <utility>

#include "philox.h"
#include "sim_types.h"
#include "sim_core.cuh"
#include "sim_warp.cuh"
#include "sim_lane.cuh"
#include "kernels.h"

namespace mbg {

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_hash(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, false>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_coop_hash(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<true, false>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_full_hash(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, true>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 2) mbg_sim_lane_coop_full_hash(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<true, true>(p, smem);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_global_hash(const SimParams p) {
    sim_lane_body<false, false>(p, p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_global_full_hash(const SimParams p) {
    sim_lane_body<false, true>(p, p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes);
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_split_hash(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, false>(p, smem,
                                reinterpret_cast<unsigned*>(p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes));
}

extern "C" __global__ void __launch_bounds__(256, 3) mbg_sim_lane_split_full_hash(const SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    sim_lane_body<false, true>(p, smem,
                               reinterpret_cast<unsigned*>(p.lane_state + (size_t)blockIdx.x * p.lane_block_bytes));
}

const void* sim_kernel_hash(int kernel, bool variant) {
    switch (kernel) {
        case 8: return variant ? (const void*)mbg_sim_lane_split_full_hash : (const void*)mbg_sim_lane_split_hash;
        case 6: return variant ? (const void*)mbg_sim_lane_global_full_hash : (const void*)mbg_sim_lane_global_hash;
        case 0: return variant ? (const void*)mbg_sim_lane_coop_hash : (const void*)mbg_sim_lane_hash;
        case 4: return variant ? (const void*)mbg_sim_lane_coop_full_hash : (const void*)mbg_sim_lane_full_hash;
        default: return nullptr;  // the warp layout and the batched kernels use the dense tables only
    }
}

}  // namespace mbg
