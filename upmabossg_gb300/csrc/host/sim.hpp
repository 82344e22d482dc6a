// Simulation handle internals (behind the opaque mbg_sim of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../../include/mbg.h"
#include "sim_host.hpp"

namespace mbg {

struct FixedPoint {
    std::vector<uint32_t> words;
    uint64_t count = 0;
};

class Sim {
public:
    ~Sim();
    void create(const CompiledModel& cm, const std::vector<std::string>& names, const mbg_sim_opts& o);
    void run(cudaStream_t stream);
    void fetch();  // copies results to the host vectors below
    // Chooses kernel, block size, shared memory and grid for a layout (update: the lane layout's
    // reader update, mbg_sim_opts::lane_update).
    void setup_layout(int layout, int block, int update = 0);
    // AUTO layout: times every layout and shape on a pilot subset once per model size class.
    void autotune();

    CompiledModel cm;
    std::vector<std::string> names;
    mbg_sim_opts opts{};
    uint64_t n_traj = 0, seed = 0;
    int device = 0, sms = 0, layout = 0, grid = 0, block = 256;
    size_t smem = 0;
    bool cached_index = false;
    bool lane_coop = true;
    bool lane_full = false;  // palette rates or nodes over 12 regulators: the `_full` lane kernels
    bool lane_split = false;  // lane layout with the active-word rows in global memory (lane_update 2)
    double jit_ms = 0;
    void* thread_kernel = nullptr;
    void* thread_kernel_hash = nullptr;  // the thread layout's window-hash variant, compiled on first use
    unsigned char* lane_state = nullptr;  // every resident block's rows (global-row lane layout), or
                                          // its active-word rows (lane_update 2)
    uint64_t lane_state_bytes = 0;
    DeviceLayout dl;
    SimParams prm{};
    uint32_t fp_capacity = 0, n_slots = 0;
    unsigned* slot_rep = nullptr;
    unsigned* slot_cnt = nullptr;
    unsigned* fp_out_states = nullptr;
    unsigned* fp_out_cnt = nullptr;
    unsigned* fp_unique = nullptr;
    void* host_small = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
    std::vector<void*> owned;

    // Window sums: the dense windows x 2^n_out table, or (hash_bits > 0) the window hash table of
    // 2^hash_bits slots (SimParams::hslots). Both are re-sized between runs, so they are owned
    // here rather than in `owned`.
    uint64_t n_bins = 0;               // windows << n_out
    int hash_bits = 0;
    unsigned long long* dense_hist = nullptr;
    unsigned long long* hslots = nullptr;
    int window_reruns = 0;             // runs repeated with a larger hash table by the last mbg_sim_run
    int pending_hash_bits = 0;         // > 0: the next run starts on a hash table of this size
    void choose_window_table();        // at create: dense or hash (mbg_sim_opts::window_table)
    void set_window_table(int bits);   // 0: dense; allocates the table and points prm at it
    void grow_window_table(int bits);  // hash table of 2^bits slots, or dense when that is smaller
    void launch(cudaStream_t stream);  // one attempt of mbg_sim_run: clear, simulate, aggregate
    // Compaction scratch (window_table.cu), allocated at the first read-back of a large table.
    unsigned* wc_bitmap = nullptr;
    unsigned* wc_wpre = nullptr;
    unsigned* wc_chunk = nullptr;
    unsigned long long* wc_total = nullptr;
    unsigned* wc_bin = nullptr;
    unsigned long long* wc_sum = nullptr;
    uint64_t wc_cap = 0;
    unsigned* fc_state = nullptr;      // compacted final states and their counts
    unsigned* fc_count = nullptr;
    uint64_t fc_cap = 0;
    void compaction_scratch();         // allocates wc_bitmap .. wc_total for n_bins (>= 2^n_out) entries

    bool ran = false, fetched = false;
    mbg_run_summary summary{};
    // Non-zero window bins in increasing order (bin = window << n_out | output state) with their
    // sums (time x 2^32, or counts); entries of window w are [wstart[w], wstart[w + 1]).
    std::vector<uint32_t> wbin;
    std::vector<uint64_t> wsum;
    std::vector<size_t> wstart;
    std::vector<uint64_t> th;
    // Reached final output states in increasing order and their trajectory counts.
    std::vector<uint32_t> fin_state;
    std::vector<uint32_t> fin_count;
    std::vector<FixedPoint> fixed;
};

// Output formats (output.cpp).
void write_probtraj_csv(const Sim& s, const std::string& path);
void write_fp_csv(const Sim& s, const std::string& path);
void write_final_states_csv(const Sim& s, const std::string& path);
void print_results(const Sim& s, std::ostream& os);
double window_prob(const Sim& s, uint64_t sum);  // probability of a window bin with this sum
double window_th(const Sim& s, int w);
std::string state_string(const std::vector<std::string>& names, const std::vector<uint32_t>& words, int n);
std::string out_state_string(const Sim& s, uint32_t idx);

}  // namespace mbg
