// Batched sweeps: many independent instances in one persistent launch, captured in a CUDA graph.
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

    ~Batch();
    void create(const std::vector<const CompiledModel*>& models, const std::vector<uint64_t>& n_traj,
                const std::vector<uint64_t>& seeds, const mbg_batch_opts& o);
    // Launch shape; rebuilds the graph.
    void configure(int block, bool cached_index, int blocks_per_sm);
    void autotune();
    void run(cudaStream_t stream);
    void fetch(int i);

    std::vector<Inst> inst;
    mbg_batch_opts opts{};
    int device = 0, sms = 0, block = 256, grid = 0, max_n = 0;
    bool cached_index = true;
    size_t smem = 0;
    unsigned slice_bytes = 0;
    uint64_t total_traj = 0;
    BatchDesc desc{};
    SimParams* d_params = nullptr;
    FpSlots* d_fps = nullptr;
    unsigned long long* d_prefix = nullptr;
    void* result_arena = nullptr;
    size_t result_bytes = 0;
    void* rep_arena = nullptr;
    size_t rep_bytes = 0;
    char* small_dev = nullptr;
    size_t small_bytes = 0;
    char* small_host = nullptr;
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
    std::vector<void*> owned;
    bool ran = false;
    mbg_run_summary summary{};
    double tune_ms[3][2] = {};

private:
    void build_graph();
};

}  // namespace mbg
