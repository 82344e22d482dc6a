/* Host FP64 Gillespie oracle: TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker for the GPU simulator. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it; the product library never links or calls it.
 *
 * It restates the reference's simulation path on the CPU in double precision:
 *   Gillespie loop, fixed point, clamp, record order   src/jit_kernels/simulation.cu:77-164
 *   node pick (first i whose prefix passes r)           src/jit_kernels/simulation.cu:9-21
 *   rate semantics (rate_down if on, rate_up if off)    src/generator.cpp:84-122
 *   transition entropy over output nodes                src/generator.cpp:146-175
 *   window split of each time slice, normalisation      src/jit_kernels/window_average_small.cu:64-93,
 *                                                       src/statistics/window_average_small.cpp:126-140
 *   discrete-time windows                               src/jit_kernels/window_average_small.cu:101-136
 *   final states / fixed points                         src/jit_kernels/final_states.cu:17-20,
 *                                                       src/statistics/fixed_states.cu:26-33,118-124
 * with the simulator's Philox4x32-10 streams in place of curand XORWOW, so the GPU path can be
 * compared trajectory by trajectory. It shares no code with the product: its parser, expression
 * evaluation, Philox and fixed-point rules are its own (front.h), and rates are evaluated from
 * its own expression trees, not from the GPU path's truth tables. The node pick uses the same exact fixed-point prefix rule as
 * the GPU path and, beside it, the FP64 prefix rule; steps where the two disagree are counted as
 * pick ties. Final steps whose FP64 time lands within 1e-6 relative of max_time are counted as
 * time ties (an FP32 dt may land on the other side).
 */
#ifndef MBG_ORACLE_H
#define MBG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_result orc_result;

typedef struct {
    uint64_t n_traj;     /* 0: sample_count of the cfg */
    uint64_t traj_base;  /* id of the first trajectory */
    uint64_t seed;
    int use_cfg_seed;    /* 1: seed_pseudorandom of the cfg */
    int frac_bits;       /* fixed-point fraction bits of the pick; 0: the compiled model's own */
    int threads;         /* 0: hardware concurrency */
    uint32_t max_steps;  /* 0: unlimited */
    int keep_trajectories; /* store per-trajectory end records */
    uint32_t redraw_period; /* 0: exact Gillespie. 99: the reference's launch segments, in which every
                            99th step draws its holding time without a flip */
    int legacy_final;    /* final-state histogram after one more flip: the rule of the earlier
                            MaBoSSG build that produced the reference's test/*.res goldens (the
                            current simulation.cu:143-147 ends before that flip) */
} orc_opts;

/* Runs the oracle on .bnd/.cfg texts. Returns NULL on error (message in err). */
orc_result* orc_run(const char* bnd_text, const char* cfg_text, const orc_opts* opts, char* err, size_t errlen);
void orc_free(orc_result* r);

/* Dimensions: n nodes, words, n_out, windows. */
void orc_dims(const orc_result* r, int* n, int* words, int* n_out, int* windows);
/* Counters: transitions, finished, fixed, step_limit, pick_ties, time_ties, steps. */
void orc_counters(const orc_result* r, uint64_t* out7);
/* Sparse window histogram: nnz entries of (window, out_state, time sum or count). */
size_t orc_hist_nnz(const orc_result* r);
void orc_hist_get(const orc_result* r, uint32_t* window, uint32_t* state, double* value);
/* Per-window sum of TH x time (continuous) or TH (discrete): `windows` doubles. */
void orc_th(const orc_result* r, double* th);
/* Final-state histogram over output states: 2^n_out counts. */
void orc_final(const orc_result* r, double* counts);
/* Per-trajectory records (keep_trajectories): states n_traj x words, time, transitions, status,
 * tie flags (bit 0 pick tie, bit 1 time tie). */
void orc_trajectories(const orc_result* r, uint32_t* states, double* times, uint32_t* transitions,
                      uint8_t* status, uint8_t* ties);
/* Elapsed wall seconds of the simulation (parse and setup excluded) and threads used. */
double orc_seconds(const orc_result* r);
int orc_threads(const orc_result* r);

/* Philox4x32-10 for known-answer tests: out = philox(ctr[4], key[2]). */
void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif
