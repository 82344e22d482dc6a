// Internal host-side interfaces of libmbg (not part of the C ABI).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../device/sim_types.h"
#include "model.hpp"

namespace mbg {

// Error classes mapped to mbg_status by the C ABI (parse errors are plain mbg::Error).
struct ArgError : Error { using Error::Error; };
struct ModelError : Error { using Error::Error; };
struct CudaError : Error { using Error::Error; };
struct NoMemError : Error { using Error::Error; };
struct DeviceError : Error { using Error::Error; };
struct StateError : Error { using Error::Error; };
struct JitError : Error { using Error::Error; };
struct IoError : Error { using Error::Error; };

// Device image of a compiled model: the arrays SimParams points at, before upload.
struct DeviceLayout {
    std::vector<DevNode> nodes;
    std::vector<LaneNode> lnodes;
    std::vector<LaneWide> lwide;
    std::vector<uint16_t> regs;
    std::vector<uint32_t> tabs;
    std::vector<uint8_t> pidx;
    std::vector<uint64_t> palette;
    std::vector<uint32_t> dep_off;
    std::vector<uint32_t> deps;  // (d << 16) | (k_d << 8) | position of the source node (0xFF: itself)
    std::vector<uint16_t> out_nodes;
    std::vector<int16_t> out_pos;
    std::vector<uint32_t> istate_thr;
    std::vector<uint32_t> tab_off, pal_off;  // per node
};

DeviceLayout layout_model(const CompiledModel& cm);
// Checks every index the kernels read out of a layout against the array it indexes (node ids,
// regulator ids, dependency entries, table, palette and side-record offsets); throws an Error
// (ModelError) naming the first one out of range. Runs on the host before any upload.
void check_layout(const CompiledModel& cm, const DeviceLayout& d);
// Model-dependent SimParams fields (sizes, clock, rate scale).
void set_model_constants(SimParams& prm, const CompiledModel& cm);
// Most trajectories one run (or one batched instance) may hold: the fixed-point buffer has one
// entry per trajectory and its hash table twice as many slots, counted in 32 bits.
constexpr uint64_t kMaxTrajectories = 1ull << 30;

// Throws if a run of n_traj trajectories of cm exceeds the result representation.
void check_model_limits(const CompiledModel& cm, uint64_t n_traj);

// Slots of the fixed-point hash table for `capacity` entries: a power of two of at least twice
// the capacity (load factor <= 1/2, so a probe always ends) and at least 1024. Throws ArgError
// for a capacity above kMaxTrajectories, whose slot count would not fit in 32 bits.
uint32_t fp_slot_count(uint64_t capacity);

// NVRTC source of the thread-per-trajectory kernel `mbg_sim_thread` specialised to one model.
std::string generate_thread_model(const CompiledModel& cm, const DeviceLayout& dl);

// Compiles (or fetches from the in-process / on-disk cache) the full NVRTC program made of the
// shared device headers and `model_src`, loads it on the current device and returns the kernel
// handle usable with cudaLaunchKernel. `compile_ms` is 0 on a cache hit. Throws mbg::Error.
// Directory of the on-disk caches (compiled kernels, tuned launch shapes): MBG_JIT_CACHE, default
// ~/.cache/mbg_gb300; cache_mkdirs creates it.
std::string cache_dir();
void cache_mkdirs(const std::string& dir);
// `window_hash`: the variant whose window sums go to the window hash table.
void* jit_thread_kernel(const std::string& model_src, double& compile_ms, bool window_hash = false);
// Compiles without loading (no device needed); returns milliseconds. Throws JitError.
double jit_compile_only(const std::string& model_src);

}  // namespace mbg
