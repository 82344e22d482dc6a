// Plain data shared by the host library, the AOT kernels and the NVRTC-compiled kernels.
// Includes nothing so that it can be pasted into an NVRTC program as is.
#pragma once

namespace mbg {

// Trajectory end states. The first three match src/trajectory_status.h:3-8.
enum TrajStatus : unsigned char {
    TRAJ_CONTINUE = 0,
    TRAJ_FINISHED = 1,
    TRAJ_FIXED_POINT = 2,
    TRAJ_STEP_LIMIT = 3,  // hit the per-trajectory step cap
    TRAJ_ERROR = 4,       // a device-side consistency check failed
};

// Device error bits (SimParams::error_flag).
enum DevError : unsigned int {
    DEV_ERR_PICK = 1u,         // no node satisfied the prefix test
    DEV_ERR_FP_OVERFLOW = 2u,  // fixed-point buffer full
    DEV_ERR_SMEM = 4u,         // launch shape does not match the model
    DEV_ERR_WINDOW_TABLE = 8u, // window hash table: an insertion ran past the probe limit (the host
                               // re-runs with a larger table; results are independent of the table)
};

// Indices into SimParams::counters.
enum Counter {
    CNT_WORK = 0,         // next trajectory to start (work queue)
    CNT_TRANSITIONS = 1,  // accepted transitions
    CNT_FINISHED = 2,
    CNT_FIXED = 3,
    CNT_STEP_LIMIT = 4,
    CNT_ERROR = 5,
    CNT_STEPS = 6,        // loop iterations (transitions + terminal steps)
    CNT_WIN_ENTRIES = 7,  // window hash table: occupied slots (distinct (window, output state) bins)
    CNT_COUNT = 8,
};

// One node of the compiled model, 64 bytes (one aligned pair of 32-byte sectors). The first 16
// bytes are all the warp layout's leaf pick reads; a truth table of up to 64 bits (k <= 5) is
// stored inline so evaluating such a node needs no second dependent load.
constexpr int kInlineRegs = 12;
struct DevNode {
    unsigned long long up, down;  // BINARY fixed-point rates
    unsigned int tab_off;         // BINARY: word offset into tabs; PALETTE: byte offset into pidx
    unsigned int pal_off;         // PALETTE: offset into palette
    unsigned short k;             // number of regulators (the node itself excluded)
    unsigned short kind;          // 0 binary, 1 palette
    unsigned int reg_off;         // offset of all k regulators in regs
    unsigned short r[kInlineRegs];  // the first min(k, 12) regulators
    unsigned long long table;     // BINARY with k <= 5: the 2^(k+1) table bits
};

// The lane layout's per-node record, 32 bytes (one sector): everything a step reads about a
// node whose rate is a two-valued table over at most 4 regulators. A two-valued node over 5..12
// regulators adds one 32-byte LaneWide entry; other nodes carry a flag and are read from their
// DevNode.
constexpr unsigned kLaneWideTable = 1u;  // 5..12 regulators: `table` indexes the LaneWide entries
constexpr unsigned kLanePalette = 2u;    // multi-valued rate: DevNode palette path
constexpr unsigned kLaneFar = 4u;        // more than 12 regulators: table and regulators in DevNode
struct LaneNode {
    unsigned long long up, down;  // fixed-point rates (BINARY)
    unsigned int table;           // k <= 4: the 2^(k+1) table bits; kLaneWideTable: LaneWide index
    unsigned short r[4];          // the first min(k, 4) regulators
    unsigned short k;             // number of regulators
    unsigned short flags;         // kLaneWideTable | kLanePalette | kLaneFar
};
struct LaneWide {
    unsigned short r[8];  // regulators 4 .. k-1
    unsigned int table[4];  // k <= 6: the 2^(k+1) table bits; k > 6: table[0] = word offset into tabs
};

struct SimParams {
    // model
    const DevNode* nodes;
    const LaneNode* lnodes;
    const LaneWide* lwide;
    const unsigned short* regs;
    const unsigned int* tabs;
    const unsigned char* pidx;
    const unsigned long long* palette;
    const unsigned int* dep_off;  // n + 1
    // For node k: every node d whose rate reads k, plus k itself, as
    // (d << 16) | (out_d << 15) | (k_d << 8) | pos: out_d = d is an output node, k_d = number of
    // regulators of d (< 128), pos = position of k among them (0xFF for d == k).
    const unsigned int* deps;
    const unsigned short* out_nodes;  // n_out
    const short* out_pos;             // n: position among outputs or -1
    const unsigned int* istate_thr;   // n
    int n, words, n_out, windows;
    int frac_bits, discrete;
    int has_palette;                 // any NODE_PALETTE node
    // Clock: unsigned fixed point with time_bits fraction bits (32 <= time_bits <= 40), so the
    // step loop needs no FP64 arithmetic (GB300's FP64 rate is a small fraction of its FP32 rate).
    int time_bits;
    unsigned long long max_time_fx, tick_fx;
    double max_time, tick;
    float to_real;  // 2^-frac_bits
    unsigned int max_steps;
    // The reference's launch segments, on request (0: off): every redraw_period-th step of a
    // trajectory draws its holding time but does not flip (thread and warp layouts).
    unsigned int redraw_period;
    unsigned long long seed;
    unsigned long long n_traj;       // trajectories of this launch
    unsigned long long traj_base;    // id of the first trajectory (Philox key part)
    // results
    unsigned long long* hist;        // windows x 2^n_out, time x 2^32 (counts if discrete)
    unsigned long long* th_hist;     // windows, TH x time x 2^32 (TH x 2^32 if discrete)
    // With hash_bits > 0 the window sums go to an open-addressed hash table instead of `hist`:
    // 2^hash_bits slots of two u64, [2i] the key (bin + 1, bin = window << n_out | output state;
    // 0 = empty) and [2i + 1] the sum; linear probing from the key's multiplicative hash.
    unsigned long long* hslots;
    int hash_bits;
    unsigned int* final_hist;        // 2^n_out
    unsigned int* fp_states;         // fp_capacity x words
    unsigned int* fp_count;
    unsigned int fp_capacity;
    unsigned int* traj_state;        // optional, n_traj x words
    double* traj_time;               // optional
    unsigned int* traj_transitions;  // optional
    unsigned char* traj_status;      // optional
    unsigned long long* counters;    // CNT_COUNT
    unsigned int* error_flag;
    // Lane layout with its per-trajectory rows in global memory (MBG_LAYOUT_LANE_GLOBAL): block b's
    // rows start at lane_state + b * lane_block_bytes.
    unsigned char* lane_state;
    unsigned long long lane_block_bytes;
};

// A batched launch over many instances (sim_warp.cuh: sim_warp_batch_body).
struct BatchDesc {
    const SimParams* params;           // n_inst
    const unsigned long long* prefix;  // n_inst + 1 cumulative trajectory counts
    int n_inst;
    unsigned long long* work;          // work-item counter
    unsigned slice_bytes;              // warp layout, per warp: SimParams copy (16-byte padded) + largest slice
    int rows;                          // lane layout: 32-node groups of the largest instance
    unsigned char* lane_state;         // lane layout with global rows: block b's rows at
    unsigned long long lane_block_bytes;  // lane_state + b * lane_block_bytes
};

// Fixed-point hash table and compacted output of one batched instance.
struct FpSlots {
    unsigned int* slot_rep;   // n_slots, 0xFFFFFFFF = empty
    unsigned int* slot_cnt;   // n_slots
    unsigned int n_slots;     // power of two, >= 2 x fp_capacity
    unsigned int* out_states; // fp_capacity x words
    unsigned int* out_cnt;    // fp_capacity
    unsigned int* n_unique;
};

}  // namespace mbg
