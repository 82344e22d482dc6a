// Host-callable launchers of the ahead-of-time kernels (sim_aot.cu, window_table.cu).
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "sim_types.h"

namespace mbg {

cudaError_t launch_sim_warp(const SimParams& p, bool cached_index, int grid, int block, size_t smem,
                            cudaStream_t stream);
cudaError_t sim_warp_configure(bool cached_index, size_t smem);
unsigned sim_warp_smem_per_warp(int n, bool cached_index);
cudaError_t sim_warp_occupancy(bool cached_index, int block, size_t smem, int* blocks_per_sm);
// `full`: the model has multi-valued rates or nodes over more than 12 regulators (the `_full`
// kernels); otherwise the kernels without those paths run.
cudaError_t launch_sim_lane(const SimParams& p, bool coop, bool full, int grid, int block, size_t smem,
                            cudaStream_t stream);
cudaError_t sim_lane_configure(bool coop, bool full, size_t smem, int block, int* blocks_per_sm);
// The lane layout with its rows in global memory (SimParams::lane_state; per-lane reader update):
// carve-out all L1, occupancy without dynamic shared memory; the launcher picks the window-hash
// twin when SimParams::hash_bits > 0. sim_kernel_limits numbers it 6 (variant: `_full`).
cudaError_t sim_lane_global_configure(bool full, int block, int* blocks_per_sm);
cudaError_t launch_sim_lane_global(const SimParams& p, bool full, int grid, int block, cudaStream_t stream);
// Dynamic shared memory of a lane-layout block (the same for both reader-update variants).
size_t sim_lane_smem(int n, int block);
// Lane layout with the active-word rows in global memory (SimParams::lane_state, G x block words
// per block at lane_block_bytes; per-lane reader update): shared memory per block, configuration,
// launch (the window-hash twin when SimParams::hash_bits > 0). sim_kernel_limits numbers it 8
// (variant: `_full`).
size_t sim_lane_split_smem(int n, int block);
cudaError_t sim_lane_split_configure(bool full, size_t smem, int block, int* blocks_per_sm);
cudaError_t launch_sim_lane_split(const SimParams& p, bool full, int grid, int block, size_t smem,
                                  cudaStream_t stream);
// The batched form (BatchDesc::lane_state); sim_kernel_limits numbers it 9 (variant: `_full`).
cudaError_t sim_lane_batch_split_configure(bool full, size_t smem, int block, int* blocks_per_sm);
cudaError_t launch_sim_lane_batch_split(const BatchDesc& b, bool full, int grid, int block, size_t smem,
                                        cudaStream_t stream);
int sim_lane_rows(int n);                 // BatchDesc::rows for models of up to n nodes
// Re-applies the attributes of a simulation kernel for the launch shapes that are about to use it
// (kernel 0: mbg_sim_lane[_coop], 1: mbg_sim_lane_batch[_coop], 2: mbg_sim_warp_batch[_gather],
// 3: mbg_sim_warp[_gather], 4: mbg_sim_lane[_coop]_full, 5: mbg_sim_lane_batch[_coop]_full,
// 6: mbg_sim_lane_global[_full], 7: mbg_sim_lane_batch_global[_full], 8: mbg_sim_lane_split[_full],
// 9: mbg_sim_lane_batch_split[_full];
// variant selects the second name; hash: the window-hash twin of kernel 0, 4, 6 or 8): kernel attributes
// are process-wide, so another handle may have changed them since this one was configured.
cudaError_t sim_kernel_limits(int kernel, bool variant, const int* blocks, const size_t* smems, const int* want,
                              int count, bool hash = false);
// The window-hash twins of the lane-layout single-simulation kernels (sim_aot_hash.cu), by the
// numbering of sim_kernel_limits (0, 4, 6, 8); the launchers pick them when SimParams::hash_bits > 0.
// The warp layout has none: it runs on the dense window table only.
const void* sim_kernel_hash(int kernel, bool variant);
std::mutex& kernel_attr_mutex();
cudaError_t launch_sim_lane_batch(const BatchDesc& b, bool coop, bool full, int grid, int block, size_t smem,
                                  cudaStream_t stream);
cudaError_t sim_lane_batch_configure(bool coop, bool full, size_t smem, int block, int* blocks_per_sm);
// Batched lane layout with global rows (BatchDesc::lane_state, lane_block_bytes; per-lane reader
// update); sim_kernel_limits numbers it 7 (variant: `_full`).
cudaError_t launch_sim_lane_batch_global(const BatchDesc& b, bool full, int grid, int block, cudaStream_t stream);
cudaError_t sim_lane_batch_global_configure(bool full, int block, int* blocks_per_sm);
cudaError_t launch_sim_warp_batch(const BatchDesc& b, bool cached_index, int grid, int block, size_t smem,
                                  cudaStream_t stream);
cudaError_t sim_warp_batch_configure(bool cached_index, size_t smem, int block, int* blocks_per_sm);
unsigned sim_warp_batch_slice_bytes(int max_n, bool cached_index);
cudaError_t launch_fp_aggregate_batch(const SimParams* params, const FpSlots* fps, int n_inst, int blocks_x,
                                      cudaStream_t stream);
cudaError_t launch_fp_aggregate(const unsigned* fp_states, const unsigned* fp_count, unsigned capacity, int words,
                                unsigned* slot_rep, unsigned* slot_cnt, unsigned n_slots, unsigned* out_states,
                                unsigned* out_cnt, unsigned* n_unique, unsigned* error_flag, int sms,
                                cudaStream_t stream);

// Window-sum compaction (window_table.cu) over n_bins = windows << n_out bins, from the dense
// table `hist` (hash_bits == 0) or the hash table `hslots` (2^hash_bits slots). Count pass: marks
// the occupied bins in `bitmap` (window_bitmap_words u32), the per-word prefixes in `wpre` (as
// many) and the per-chunk prefixes in `chunk` (window_chunks u32); *total = occupied bins. Emit
// pass (after the count pass, with out_bin / out_sum holding *total entries): the (bin, sum)
// pairs in increasing bin order.
unsigned long long window_bitmap_words(unsigned long long n_bins);
unsigned window_chunks(unsigned long long n_bins);
cudaError_t launch_window_count(const unsigned long long* hist, const unsigned long long* hslots, int hash_bits,
                                unsigned long long n_bins, unsigned* bitmap, unsigned* wpre, unsigned* chunk,
                                unsigned long long* total, int sms, cudaStream_t stream);
cudaError_t launch_window_emit(const unsigned long long* hist, const unsigned long long* hslots, int hash_bits,
                               unsigned long long n_bins, const unsigned* bitmap, const unsigned* wpre,
                               const unsigned* chunk, unsigned* out_bin, unsigned long long* out_sum, int sms,
                               cudaStream_t stream);
// One window of many batched instances: span i copies n u64 sums from src to out + dst. Spans in
// device memory; max_n the largest n.
struct WindowSpan {
    const unsigned long long* src;
    unsigned long long dst;
    unsigned long long n;
};
cudaError_t launch_window_gather(const WindowSpan* spans, int n_spans, unsigned long long max_n,
                                 unsigned long long* out, cudaStream_t stream);
// The same two passes over the dense 2^n_out final-state counts (n_states entries): out_state /
// out_count get the reached output states in increasing order and their counts. The scratch
// arrays are those of the window compaction, sized for n_states or more.
cudaError_t launch_final_count(const unsigned* counts, unsigned long long n_states, unsigned* bitmap,
                               unsigned* wpre, unsigned* chunk, unsigned long long* total, int sms,
                               cudaStream_t stream);
cudaError_t launch_final_emit(const unsigned* counts, unsigned long long n_states, const unsigned* bitmap,
                              const unsigned* wpre, const unsigned* chunk, unsigned* out_state, unsigned* out_count,
                              int sms, cudaStream_t stream);

}  // namespace mbg
