// Batched sweeps: many independent instances, grouped by model size into classes; each class is one
// persistent launch (lane or warp layout, its own shape), and the whole batch is one CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../../include/mbg.h"
#include "sim_host.hpp"

namespace mbg {

class Batch {
public:
    struct Inst {
        CompiledModel cm;
        uint64_t n_traj = 0, seed = 0;
        int cls = 0;           // size class
        SimParams prm{};
        FpSlots fp{};
        size_t small_off = 0;  // offset of this instance's counters in the small block
        // host results
        bool fetched = false;
        std::vector<uint64_t> hist, th;
        std::vector<uint32_t> fin;
        std::vector<uint32_t> fp_words, fp_cnt;
        mbg_run_summary summary{};
    };

    // Instances of one size class and the launch that runs them.
    struct Class {
        int max_n = 0;                      // nodes of the largest member
        bool full = false;                  // a member has palette rates or nodes over 12 regulators
        std::vector<int> members;           // instance indices, ascending
        uint64_t traj = 0;                  // trajectories of all members
        size_t first = 0;                   // position of the first member in the class-ordered arrays
        BatchDesc desc{};                   // work over all members' trajectories
        BatchDesc pilot{};                  // a subset of every member's trajectories, for timing shapes
        BatchDesc pilot_long{};             // four times the pilot, for re-timing the closest shapes
        bool has_long = false;              // pilot_long covers more than the pilot
        int layout = MBG_LAYOUT_LANE;       // MBG_LAYOUT_LANE, MBG_LAYOUT_LANE_GLOBAL or MBG_LAYOUT_WARP
        int block = 128;
        int variant = 0;                    // lane: 0 per-lane reader update, 1 cooperative, 2 per-lane with
                                            // the active words in global memory; warp: 1 regulator index cache
        size_t smem = 0;
        int grid = 0;
        void* lane_buf = nullptr;           // global rows (MBG_LAYOUT_LANE_GLOBAL) or active-word rows (lane
                                            // variant 2) of the resident blocks
        size_t lane_buf_bytes = 0;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaStream_t stream = nullptr;      // the class's branch of the graph
        cudaEvent_t join = nullptr;         // end of that branch
        float kernel_ms = 0.f;
        std::vector<mbg_batch_class_timing> timings;  // every shape the autotuner timed
    };

    ~Batch();
    void create(const std::vector<const CompiledModel*>& models, const std::vector<uint64_t>& n_traj,
                const std::vector<uint64_t>& seeds, const mbg_batch_opts& o);
    // Launch shape of class c (no graph rebuild).
    void configure(int c, int layout, int block, int variant);
    void autotune();
    void run(cudaStream_t stream);
    void fetch(int i);
    // Window w (w < 0: counted from each instance's last window) of every instance, gathered on the
    // device into one array: instance i's 2^outputs sums after those of the instances before it.
    void window_sums(int w, std::vector<uint64_t>& out);

    std::vector<Inst> inst;
    std::vector<Class> classes;
    mbg_batch_opts opts{};
    int device = 0, sms = 0;
    uint64_t total_traj = 0;
    SimParams* d_params = nullptr;  // class order
    FpSlots* d_fps = nullptr;       // class order
    void* result_arena = nullptr;
    size_t result_bytes = 0;
    void* rep_arena = nullptr;
    size_t rep_bytes = 0;
    char* small_dev = nullptr;
    size_t small_bytes = 0;
    char* small_host = nullptr;
    cudaStream_t capture_stream = nullptr;
    cudaEvent_t fork = nullptr;             // start of the class branches
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void*> owned;
    bool ran = false, tuned = false;
    mbg_run_summary summary{};

private:
    void build_graph();
    void apply_limits();
    cudaError_t launch_class(const Class& k, const BatchDesc& d, cudaStream_t s) const;
};

// Size class of a model with n nodes: c = ceil(log2(ceil(n / 32))), so class c holds models of at
// most 32 * 2^c nodes (c = 0 .. 6), class 7 everything larger than 4096 nodes. The lane layout's
// shared memory grows with a class's largest model, so narrow classes keep occupancy up.
int batch_size_class(int n);

}  // namespace mbg
