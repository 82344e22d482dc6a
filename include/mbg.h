/* MaBoSS-style continuous-time Boolean network simulator for one NVIDIA GB300 (sm_103a).
 *
 * C ABI of libmbg.so: plain pointers and sizes, status codes, caller-owned handles. The
 * `MaBoSSG` command line is a thin client of this interface. Reference interfaces replaced
 * (paths inside DominicJW/UPMaBoSSG):
 *
 *   mbg_model_parse_files / _strings  driver::parse, src/parser/driver.cpp:16-31 (+ parse_one 33-43)
 *   mbg_model_info                    main.cpp:128-152 (cfg constants, output mask and limits)
 *   mbg_sim_create                    kernel_compiler::compile_simulation, src/kernel_compiler.cpp:61-164,
 *                                     simulation_runner ctor, src/simulation_runner.cu:42-52, and the
 *                                     stats constructors, main.cpp:60-74
 *   mbg_sim_run                       simulation_runner::run_simulation, src/simulation_runner.cu:54-180,
 *                                     and stats_composite::finalize, src/statistics/stats_composite.cpp:14
 *   mbg_sim_probtraj                  window_average_small_stats::finalize + get_single_result_prob,
 *                                     src/statistics/window_average_small.cpp:91-140
 *   mbg_sim_final_states              final_states_stats::finalize, src/statistics/final_states.cpp:45-51
 *   mbg_sim_fixed_points              fixed_states_stats result map, src/statistics/fixed_states.cu:118-124
 *   mbg_write_probtraj_csv            window_average_small_stats::write_csv, window_average_small.cpp:181-250
 *   mbg_write_fp_csv                  fixed_states_stats::write_csv, src/statistics/fixed_states.cu:154-187
 *   mbg_print_results                 stats_composite::visualize (final, fixed, window order of main.cpp:65-74)
 *
 * Every call returns a status; nothing exits or traps. Handles are not thread safe; distinct
 * handles may be used from distinct threads. Each simulation handle uses one device and the
 * stream passed to mbg_sim_run.
 */
#ifndef MBG_H
#define MBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MBG_OK = 0,
    MBG_ERR_ARG = 1,      /* invalid argument */
    MBG_ERR_IO = 2,       /* file cannot be read or written */
    MBG_ERR_PARSE = 3,    /* .bnd / .cfg syntax or semantic error */
    MBG_ERR_MODEL = 4,    /* model outside the supported limits */
    MBG_ERR_CUDA = 5,     /* CUDA runtime error or no device */
    MBG_ERR_JIT = 6,      /* NVRTC compilation failed */
    MBG_ERR_NOMEM = 7,    /* device or host allocation failed */
    MBG_ERR_DEVICE = 8,   /* a kernel reported an error flag */
    MBG_ERR_STATE = 9     /* call out of order (e.g. results before run) */
} mbg_status;

typedef struct mbg_model mbg_model;
typedef struct mbg_sim mbg_sim;

typedef struct {
    int32_t nodes;          /* N */
    int32_t words;          /* ceil(N / 32) state words */
    int32_t outputs;        /* non-internal nodes */
    int32_t windows;        /* ceil(max_time / time_tick) */
    int32_t discrete_time;  /* cfg discrete_time != 0 */
    int32_t frac_bits;      /* fixed-point fraction bits of the rates */
    int32_t max_regulators; /* largest number of nodes a rate reads */
    int32_t palette_nodes;  /* nodes with multi-valued rates */
    double max_time, time_tick;
    uint64_t sample_count, seed;
} mbg_model_info;

/* Trajectory layout: 0 auto (timed on a pilot, once per model size class), 1 thread per
 * trajectory (NVRTC-compiled evaluator, state in registers, every rate re-evaluated per step),
 * 2 warp per trajectory (table driven), 3 lane: thread per trajectory, table driven, state in
 * shared memory, rates updated incrementally, 4 lane with the per-trajectory state in global
 * memory (L1/L2-cached; for networks whose state leaves too few trajectories in shared memory).
 * All give identical results. */
enum { MBG_LAYOUT_AUTO = 0, MBG_LAYOUT_THREAD = 1, MBG_LAYOUT_WARP = 2, MBG_LAYOUT_LANE = 3, MBG_LAYOUT_LANE_GLOBAL = 4 };

typedef struct {
    uint64_t n_traj;           /* 0: cfg sample_count */
    uint64_t traj_base;        /* id of the first trajectory (Philox stream) */
    uint64_t seed;             /* used when use_cfg_seed == 0 */
    int32_t use_cfg_seed;      /* 1: cfg seed_pseudorandom (default) */
    int32_t layout;            /* MBG_LAYOUT_* */
    int32_t record_trajectories; /* keep per-trajectory end state, time, transitions, status */
    int32_t device;            /* CUDA device ordinal */
    uint32_t max_steps;        /* per-trajectory step cap; 0: none */
    int32_t block_size;        /* threads per block; 0: default */
    int32_t blocks_per_sm;     /* 0: occupancy limit */
    int32_t thread_cutoff;     /* AUTO: > 0 runs N <= cutoff thread per trajectory and the rest warp
                                  per trajectory without timing; 0: autotune */
    int32_t lane_update;       /* LANE: readers of a flipped node updated 0: warp-cooperatively
                                  (default), 1: by their own lane, 2: by their own lane with the
                                  active-node words in global memory instead of shared memory
                                  (more resident trajectories per SM where shared memory bounds
                                  them); AUTO times all three */
    int32_t window_table;      /* where the window sums accumulate: 0 auto (the dense table up to
                                  2 GiB, the faster one; the hash table beyond), 1 the dense
                                  windows x 2^outputs table (the reference's layout), 2 an
                                  open-addressed hash table of the (window, output state) bins
                                  reached, grown and re-run when full */
    int32_t window_hash_bits;  /* hash table: log2 of its initial slot count (10..31); 0 automatic */
    uint32_t redraw_period;    /* 0 (default): the exact Gillespie process. 99: the reference build's
                                  process, whose launches of at most 99 records end without a flip,
                                  the next launch drawing the same state's holding time again
                                  (src/simulation_runner.cu:51, src/jit_kernels/simulation.cu:143-147):
                                  every 99th step draws a holding time but flips nothing. For
                                  statistical comparison with that build; thread and warp layouts. */
} mbg_sim_opts;

typedef struct {
    uint64_t trajectories;     /* trajectories simulated */
    uint64_t transitions;      /* accepted flips (time < max_time) */
    uint64_t steps;            /* loop iterations, including terminal ones */
    uint64_t finished, fixed_points, step_limited, errors;
    uint64_t fixed_point_states; /* distinct fixed states */
    uint32_t device_error;     /* device error bits */
    int32_t layout;            /* layout that ran */
    double sim_ms;             /* device time of the last mbg_sim_run (CUDA events) */
    double kernel_ms;          /* device time of its simulation kernel alone */
    double jit_ms;             /* NVRTC compile time at create (0 if cached) */
    int32_t block_size;        /* threads per block of the simulation kernel */
    int32_t grid_size;         /* blocks of the simulation kernel */
    int32_t lane_update;       /* LANE: 0 cooperative, 1 per-lane reader updates, 2 per-lane with
                                  the active-node words in global memory */
    int32_t window_table;      /* 1 dense table, 2 hash table */
    int32_t window_hash_bits;  /* hash table: log2 of its slot count in the last run */
    int32_t window_reruns;     /* runs repeated with a larger hash table (results are the same) */
    uint64_t window_entries;   /* hash table: distinct (window, output state) bins reached */
} mbg_run_summary;

const char* mbg_last_error(void);
const char* mbg_version(void);
int mbg_device_count(void);

mbg_status mbg_model_parse_files(const char* bnd_path, const char* cfg_path, mbg_model** out);
mbg_status mbg_model_parse_strings(const char* bnd_text, const char* cfg_text, mbg_model** out);
/* mbg_model_parse_files followed by the cfg statements in `cfg_overrides` (NULL or "": none),
 * applied after the cfg file so that they replace its values: `$var = 2;`, `max_time = 50;`,
 * `sample_count = 1000;`, `A.istate = 1;`, `[A].istate = 0.3 [1], 0.7 [0];`. Parameter overrides
 * without editing the model files (the role of MaBoSS's `-e` configuration expressions). */
mbg_status mbg_model_parse_files_overrides(const char* bnd_path, const char* cfg_path, const char* cfg_overrides,
                                           mbg_model** out);
/* Run constants of a model built from arrays (the cfg's max_time, time_tick, sample_count,
 * seed_pseudorandom and discrete_time). */
typedef struct {
    double max_time;
    double time_tick;
    uint64_t sample_count;
    uint64_t seed;
    int32_t discrete_time;
    int32_t reserved;
} mbg_model_run;
/* A model given by arrays instead of .bnd/.cfg text (synthetic and generated networks, sweeps
 * built by a program); it replaces writing a .bnd/.cfg pair for driver::parse
 * (src/parser/driver.cpp:16-31). Node i reads regs[reg_off[i] .. reg_off[i + 1]) (n + 1 offsets,
 * reg_off[0] = 0; distinct node indices other than i, in any order, at most 24); its logic over
 * them is bit idx = sum_j state(regs[reg_off[i] + j]) << j of the words starting at
 * logic[logic_off[i]] (2^k bits for k regulators; every table must lie within the logic_words
 * words of `logic`). The node turns on at rate_up[i] while it is off
 * and its logic is 1, and off at rate_down[i] while it is on and its logic is 0: MaBoSS's
 * `rate_up = @logic ? u : 0; rate_down = @logic ? 0 : d;` (generator.cpp:84-122), compiled
 * exactly as that .bnd text would be. istate[i] in [0, 1]; is_output (NULL: every node) marks the
 * non-internal nodes; names (NULL: "N0", "N1", ...) must be distinct and non-empty. */
mbg_status mbg_model_from_arrays(int32_t n, const char* const* names, const int32_t* reg_off, const int32_t* regs,
                                 const uint32_t* logic, int64_t logic_words, const int64_t* logic_off,
                                 const double* rate_up, const double* rate_down, const double* istate,
                                 const uint8_t* is_output, const mbg_model_run* run, mbg_model** out);
void mbg_model_destroy(mbg_model* m);
mbg_status mbg_model_info_get(const mbg_model* m, mbg_model_info* out);
const char* mbg_model_node_name(const mbg_model* m, int32_t i);
/* Output node indices (node order), `cap` entries at most; returns the count. */
int32_t mbg_model_outputs(const mbg_model* m, int32_t* idx, int32_t cap);

/* Rate of node `node` in the full state `state` (one byte per node, 0 or 1), from the compiled
 * tables, host side: the exact fixed-point value and the real value. Replaces the generated
 * `<node>_rate` device functions of src/generator.cpp:84-122 as an inspectable function. */
mbg_status mbg_model_rate(const mbg_model* m, int32_t node, const uint8_t* state, uint64_t* fixed_rate,
                          double* rate);

/* A copy of `base` whose node i has its up rates multiplied by up_scale[i] and its down rates by
 * down_scale[i] (NULL: 1), re-quantized as if the cfg had carried the scaled values. For
 * parameter sweeps: no re-parse, no re-tabulation. Models with multi-valued rates are refused.
 * The copy has no expression trees (mbg_model_rate and the simulation work; nothing else needs
 * them). */
mbg_status mbg_model_with_rate_scales(const mbg_model* base, const double* up_scale, const double* down_scale,
                                      mbg_model** out);

/* Mutant analysis: a copy of `base` with node nodes[j] clamped ON (values[j] = 1) or OFF (0). A
 * clamped node starts at its value and its rate is zero wherever it holds it, so it never leaves
 * it; every other node is unchanged. The copy simulates exactly as the model whose cfg sets the
 * node's istate to the value and whose bnd sets its rate_down (ON) or rate_up (OFF) to 0. The
 * reference lists mutant analysis as future work (README.md "Next steps"). No expression trees
 * in the copy, as for mbg_model_with_rate_scales. */
mbg_status mbg_model_with_mutations(const mbg_model* base, const int32_t* nodes, const int32_t* values,
                                    int32_t count, mbg_model** out);

/* Builds the model's device tables on the host and checks every index the kernels read from them
 * (node, regulator and dependency ids, table, palette and side-record offsets) against the array
 * it indexes; MBG_ERR_MODEL names the first one out of range. Needs no GPU; mbg_sim_create and
 * mbg_batch_create run the same check before uploading. */
mbg_status mbg_model_layout_check(const mbg_model* m);

/* Generates the model's thread-per-trajectory kernel and compiles it with NVRTC for sm_103a
 * without loading it (needs no GPU). */
mbg_status mbg_model_jit_check(const mbg_model* m, double* compile_ms);

void mbg_sim_opts_default(mbg_sim_opts* o);
mbg_status mbg_sim_create(const mbg_model* m, const mbg_sim_opts* o, mbg_sim** out);
void mbg_sim_destroy(mbg_sim* s);
/* Runs all trajectories on `stream` (a cudaStream_t, NULL for the legacy stream) and waits. */
mbg_status mbg_sim_run(mbg_sim* s, void* stream);
mbg_status mbg_sim_summary(const mbg_sim* s, mbg_run_summary* out);
/* windows x 2^outputs probabilities and the per-window transition entropy, as the reference
 * reports them (time share / (n x tick), or count / n in discrete time). */
mbg_status mbg_sim_probtraj(mbg_sim* s, double* probs, double* tr_entropy);
/* Raw fixed-point sums: windows x 2^outputs (time x 2^32, or counts) and windows TH sums. */
mbg_status mbg_sim_probtraj_raw(mbg_sim* s, uint64_t* sums, uint64_t* th_sums);
/* The non-zero window bins only, in increasing order: bin = window x 2^outputs + output state,
 * with its raw sum (as mbg_sim_probtraj_raw) and probability (as mbg_sim_probtraj); any of the
 * three arrays may be NULL; `cap` entries at most, `*count` gets the number of non-zero bins. The
 * read-back for large output spaces (20 outputs: 2^20 states per window), where the dense arrays
 * are mostly zeros: only the bins the run reached leave the device. Replaces the host walk over the
 * dense table, src/statistics/window_average_small.cpp:126-140. */
mbg_status mbg_sim_probtraj_sparse(mbg_sim* s, uint64_t* bins, uint64_t* sums, double* probs, size_t cap,
                                   size_t* count);
/* 2^outputs final-state probabilities. */
mbg_status mbg_sim_final_states(mbg_sim* s, double* probs);
/* The reached final output states only, in increasing order, with their probabilities: `cap`
 * entries at most, `*count` gets their number (states or probs may be NULL). Large output spaces
 * are compacted on the device, so only the reached states leave it. The reference copies the
 * dense count array back and prints its non-zero entries (src/statistics/final_states.cpp:45-66). */
mbg_status mbg_sim_final_states_sparse(mbg_sim* s, uint64_t* states, double* probs, size_t cap, size_t* count);
/* Distinct fixed points in reference order (highest state word first): states (n x words),
 * probabilities; `cap` entries at most, `*count` gets the total. */
mbg_status mbg_sim_fixed_points(mbg_sim* s, uint32_t* states, double* probs, size_t cap, size_t* count);
/* Per-trajectory end records (record_trajectories): n_traj x words states, end times,
 * transitions and statuses (1 finished, 2 fixed point, 3 step limit, 4 error). */
mbg_status mbg_sim_trajectories(mbg_sim* s, uint32_t* states, double* times, uint32_t* transitions,
                                uint8_t* status);

mbg_status mbg_write_probtraj_csv(mbg_sim* s, const char* prefix);
mbg_status mbg_write_fp_csv(mbg_sim* s, const char* prefix);
/* <prefix>_final_states.csv: `Final States (K)`, a header `Proba\tState\t<output nodes>`, then one
 * row per reached output state (increasing index) with its share of the trajectories, its name
 * and one 0/1 column per output node. The reference prints this histogram to stdout only
 * (final_states.cpp:53-68). */
mbg_status mbg_write_final_states_csv(mbg_sim* s, const char* prefix);
/* The reference's stdout report (final points, fixed points, windows) to a file path or "-". */
mbg_status mbg_print_results(mbg_sim* s, const char* path);

/* Measured 64-bit atomic-add (reduction) throughput of device `device`'s L2: atomics per second
 * when every thread of a GPU-filling grid adds to `distinct` addresses (a power of two, at most
 * 2^26: an L2-resident table at up to 512 MiB) with no result returned, the form of the window-sum
 * flushes. No counterpart in the reference; the denominator of the flushes' roofline. */
mbg_status mbg_device_l2_atomic_rate(int32_t device, uint32_t distinct, double* atomics_per_s);

/* ---- Batched parameter sweeps --------------------------------------------------------------
 * Many independent simulations ("instances": any models, trajectory counts and seeds) grouped by
 * model size into classes (<= 32, 64, 128, ..., 4096 nodes, larger); each class is one persistent
 * launch in the lane or the warp layout with its own block size, and all classes, the fixed-point
 * aggregation and the counter read-back are captured once into a CUDA graph replayed by every
 * mbg_batch_run. Replaces one reference CLI run per instance (src/main.cpp:101-169), each of which
 * recompiles its kernels with NVRTC. Results per instance are the same as a single simulation's. */
typedef struct mbg_batch mbg_batch;

typedef struct {
    int32_t device;        /* CUDA device ordinal */
    uint32_t max_steps;    /* per-trajectory step cap; 0: none */
    int32_t block_size;    /* threads per block (multiple of 32, <= 256); 0: default or autotuned */
    int32_t blocks_per_sm; /* 0: occupancy limit */
    int32_t autotune;      /* 1: on the first run, time every shape of every class on a pilot subset
                              of its trajectories and keep the fastest per class */
    int32_t layout;        /* 0: autotuned per class (without autotune: lane where it fits);
                              MBG_LAYOUT_LANE, MBG_LAYOUT_LANE_GLOBAL or MBG_LAYOUT_WARP: that
                              layout for every class (global rows: per-lane reader update) */
    int32_t lane_variant;  /* lane layout without autotune: 0 per-lane reader update (default),
                              1 cooperative, 2 per-lane with the active-node words in global
                              memory (mbg_sim_opts::lane_update 2) */
} mbg_batch_opts;

/* One launch shape the autotuner timed for a class. */
typedef struct {
    int32_t layout;        /* MBG_LAYOUT_LANE, MBG_LAYOUT_LANE_GLOBAL or MBG_LAYOUT_WARP */
    int32_t block_size;
    int32_t variant;       /* lane: 0 per-lane reader update, 1 cooperative, 2 per-lane with the
                              active-node words in global memory; warp: 1 regulator-index cache */
    int32_t reserved;
    double kernel_ms;      /* pilot kernel time */
} mbg_batch_class_timing;

/* A size class of a batch and the launch that runs it. */
typedef struct {
    int32_t max_nodes;     /* nodes of the largest member */
    int32_t instances;
    uint64_t trajectories;
    int32_t layout, block_size, variant, grid;
    double kernel_ms;      /* device time of the class launch in the last run */
    int32_t timings;       /* shapes timed by the autotuner (mbg_batch_class_timings) */
    int32_t reserved;
} mbg_batch_class_info;

void mbg_batch_opts_default(mbg_batch_opts* o);
/* n_traj and seeds may be NULL: each instance then uses its cfg sample_count / seed_pseudorandom. */
mbg_status mbg_batch_create(const mbg_model* const* models, int32_t n_models, const uint64_t* n_traj,
                            const uint64_t* seeds, const mbg_batch_opts* o, mbg_batch** out);
void mbg_batch_destroy(mbg_batch* b);
/* Runs every instance on `stream` (NULL: an internal stream) and waits. */
mbg_status mbg_batch_run(mbg_batch* b, void* stream);
/* Totals over the batch (sim_ms: the whole graph, kernel_ms: the simulation kernel). */
mbg_status mbg_batch_summary(const mbg_batch* b, mbg_run_summary* out);
mbg_status mbg_batch_instance_summary(const mbg_batch* b, int32_t i, mbg_run_summary* out);
mbg_status mbg_batch_probtraj(mbg_batch* b, int32_t i, double* probs, double* tr_entropy);
mbg_status mbg_batch_probtraj_raw(mbg_batch* b, int32_t i, uint64_t* sums, uint64_t* th_sums);
/* One window of every instance at once (window < 0 counts from each instance's last window: -1 is
 * the final window): the instances' 2^outputs probabilities one after the other in instance order,
 * instance i's entries after those of instances 0..i-1. One gather on the device and one copy,
 * instead of a windows x 2^outputs read per instance. */
mbg_status mbg_batch_window_probs(mbg_batch* b, int32_t window, double* probs);
mbg_status mbg_batch_final_states(mbg_batch* b, int32_t i, double* probs);
mbg_status mbg_batch_fixed_points(mbg_batch* b, int32_t i, uint32_t* states, double* probs, size_t cap,
                                  size_t* count);
/* Size classes (in increasing size) and their launch shapes. */
mbg_status mbg_batch_class_count(const mbg_batch* b, int32_t* count);
mbg_status mbg_batch_class(const mbg_batch* b, int32_t c, mbg_batch_class_info* out);
/* The shapes the autotuner timed for class c: up to cap entries, *count gets their number. */
mbg_status mbg_batch_class_timings(const mbg_batch* b, int32_t c, mbg_batch_class_timing* out, int32_t cap,
                                   int32_t* count);

/* ---- Learned surrogate for sweep screening ---------------------------------------------------
 * No counterpart in the reference. An ensemble of MLPs (BF16 weights, FP32 accumulation, ReLU
 * hidden layers, softmax output) trained on simulated (parameters -> output-state distribution)
 * pairs; screening uses the ensemble mean and its spread (largest total-variation distance of a
 * member from the mean). Parameters are flattened per layer as W [in][out] row-major, then b. */
typedef struct mbg_surrogate mbg_surrogate;

mbg_status mbg_surrogate_create(int32_t in_dim, int32_t hidden, int32_t hidden_layers, int32_t out_dim,
                                int32_t ensemble, uint64_t seed, int32_t device, mbg_surrogate** out);
/* Forward products (training and prediction) on the tcgen05 tensor cores (1, default: 128x128 tiles,
 * FP32 accumulator in tensor memory) or on the mma.sync kernel (0); both compute the same BF16
 * products with FP32 accumulation (summation order differs). */
mbg_status mbg_surrogate_set_tensor_path(mbg_surrogate* s, int32_t tcgen05);
/* Device time of one forward pass of every ensemble member over `rows` rows (the GEMMs with their
 * bias/ReLU epilogues), the mean over `reps` passes timed with CUDA events: the tensor-core
 * throughput figure (2 * rows * members * sum of layer in x out FLOP per pass). */
mbg_status mbg_surrogate_time_forward(mbg_surrogate* s, int32_t rows, int32_t reps, double* ms_per_pass);
void mbg_surrogate_destroy(mbg_surrogate* s);
/* Trains every member for `epochs` passes over (x: n x in_dim, y: n x out_dim distributions) with
 * Adam, the learning rate decaying from lr along a half cosine (floored at lr / 100) over the call;
 * *last_loss gets the mean cross-entropy of the last epoch. */
mbg_status mbg_surrogate_train(mbg_surrogate* s, const float* x, const float* y, int64_t n, int32_t epochs,
                               int32_t batch, float lr, uint64_t seed, float* last_loss);
/* probs: n x out_dim ensemble-mean distributions; spread: n values (either may be NULL). */
mbg_status mbg_surrogate_predict(mbg_surrogate* s, const float* x, int64_t n, float* probs, float* spread);
/* score: n ensemble-mean probabilities of output state `column` alone; spread as above (may be
 * NULL). For screening many candidates on one target state without reading every distribution
 * back. */
mbg_status mbg_surrogate_predict_column(mbg_surrogate* s, const float* x, int64_t n, int32_t column, float* score,
                                        float* spread);
int64_t mbg_surrogate_param_count(const mbg_surrogate* s);
mbg_status mbg_surrogate_get_params(mbg_surrogate* s, int32_t member, float* params);
mbg_status mbg_surrogate_set_params(mbg_surrogate* s, int32_t member, const float* params);
/* Mean cross-entropy of member `member` on (x, y) and its gradient (param_count floats). */
mbg_status mbg_surrogate_gradients(mbg_surrogate* s, int32_t member, const float* x, const float* y,
                                   int32_t rows, float* loss, float* grads);

/* No counterpart in the reference. Fixed-point aggregation for callers that must not allocate
 * device memory (a host that owns every allocation through its own pool, a latency-critical loop
 * where cudaMalloc could stall the device, a fixed device footprint after start-up). All buffers
 * are device memory owned by the caller: `states` holds n_states x words state words;
 * `unique_states` (room for n_states x words) and `counts` (n_states) receive the distinct states
 * and how often each occurs, in no particular order; `*n_unique` their number. Nothing is
 * allocated: the hash table is a 512 KiB device array inside libmbg.so that every GPU loading the
 * library keeps until exit. At most 32768 states per call (MBG_ERR_ARG beyond). The work is queued
 * on `stream`; results are valid once the stream has completed it. The first call on a device
 * (and the first after the device's context was replaced, e.g. by cudaDeviceReset) looks the
 * array's address up on that device, so make it before any stream capture. Calls share
 * the array and each clears it first: calls queued on one stream are safe, calls that overlap on
 * the GPU race. */
mbg_status mbg_fixed_points_aggregate_noalloc(const uint32_t* states, uint32_t n_states, int32_t words,
                                              uint32_t* unique_states, uint32_t* counts, uint32_t* n_unique,
                                              void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MBG_H */
