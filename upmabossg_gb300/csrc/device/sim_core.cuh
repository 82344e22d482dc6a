// Device building blocks shared by the thread-per-trajectory kernels (NVRTC-compiled per model,
// or table driven) and the warp-per-trajectory kernel. Includes nothing: sim_types.h and
// philox.h come first in both the nvcc and the NVRTC translation unit.
//
// Per-trajectory semantics restate src/jit_kernels/simulation.cu:77-164:
//   * a state with total rate 0 is a fixed point and holds until max_time (114-118);
//   * otherwise dt = -log(U) / total (FP32 here, the clock itself is FP64), the clock is clamped
//     to max_time (129-131), and the slice [t, t+dt] is credited to the state held before the
//     flip (137-147);
//   * the trajectory ends when the clock reaches max_time (143);
//   * the flipped node is the first whose rate prefix passes the target (select_flip_bit, 9-21),
//     here with exact 64-bit fixed-point rates.
// Window accumulation restates src/jit_kernels/window_average_small.cu:64-93: a slice is split at
// the window edges w*tick and each piece is added to bin [w][output state]; the transition
// entropy is added weighted by the piece length. Consecutive slices in the same (window, state)
// are merged before they are written, so one trajectory issues about one atomic per change of
// output state. Bins are 64-bit fixed point (2^-32 time units), which makes the result independent
// of the order of the atomics.
#pragma once

namespace mbg {

#define MBG_FULL 0xffffffffu

__device__ __forceinline__ unsigned long long fixed32(double x) { return __double2ull_rn(x * 4294967296.0); }

struct WindowAcc {
    int w;          // current window
    double wend;    // end of window w
    double run_t0;  // start of the current run of one output state inside window w
    unsigned run_s; // output state of the run
    float th;       // sum of TH x length inside window w
};

__device__ __forceinline__ void win_begin(WindowAcc& a, const SimParams& p, unsigned s) {
    a.w = 0;
    a.wend = p.tick;
    a.run_t0 = 0.0;
    a.run_s = s;
    a.th = 0.f;
}

__device__ __forceinline__ void win_flush_run(WindowAcc& a, const SimParams& p, double t_end, bool leader) {
    double len = t_end - a.run_t0;
    if (leader && len > 0.0)
        atomicAdd(p.hist + (((unsigned long long)a.w << p.n_out) | a.run_s), fixed32(len));
}

__device__ __forceinline__ void win_flush_th(WindowAcc& a, const SimParams& p, bool leader) {
    if (leader && a.th != 0.f) atomicAdd(p.th_hist + a.w, fixed32((double)a.th));
    a.th = 0.f;
}

// Continuous time: the output state s with entropy h was held over [t0, t1].
__device__ __forceinline__ void win_slice(WindowAcc& a, const SimParams& p, double t0, double t1, unsigned s,
                                          float h, bool leader) {
    if (s != a.run_s) {
        win_flush_run(a, p, t0, leader);
        a.run_s = s;
        a.run_t0 = t0;
    }
    while (t1 > a.wend && a.w + 1 < p.windows) {
        a.th += h * (float)(a.wend - t0);
        win_flush_run(a, p, a.wend, leader);
        win_flush_th(a, p, leader);
        t0 = a.wend;
        a.run_t0 = t0;
        a.w += 1;
        a.wend = (double)(a.w + 1) * p.tick;
    }
    a.th += h * (float)(t1 - t0);
}

__device__ __forceinline__ void win_end(WindowAcc& a, const SimParams& p, double t_end, bool leader) {
    win_flush_run(a, p, t_end, leader);
    win_flush_th(a, p, leader);
}

// Discrete time (window_average_small.cu:101-136): one count per recorded step, in the window of
// the step's start time, which is step * tick.
__device__ __forceinline__ void win_discrete(const SimParams& p, unsigned long long step, unsigned s, float h,
                                             bool leader) {
    int w = step < (unsigned long long)p.windows ? (int)step : p.windows - 1;
    if (leader) {
        atomicAdd(p.hist + (((unsigned long long)w << p.n_out) | s), 1ull);
        if (h != 0.f) atomicAdd(p.th_hist + w, fixed32((double)h));
    }
}

// Transition entropy from the summed output rates (fixed point) and sum r*log2(r) (real units):
// -sum p log2 p = log2 R - (sum r log2 r) / R.
__device__ __forceinline__ float entropy_from_sums(unsigned long long rout, float cout, float to_real) {
    if (rout == 0ull) return 0.f;
    float R = (float)rout * to_real;
    float h = __log2f(R) - cout / R;
    return h > 0.f ? h : 0.f;
}

__device__ __forceinline__ double next_time(const SimParams& p, double t, unsigned long long step, unsigned u,
                                            unsigned long long total) {
    if (p.discrete) {
        double t1 = (double)(step + 1) * p.tick;
        return (step + 1 >= (unsigned long long)p.windows) ? p.max_time : t1;
    }
    float rate = (float)total * p.to_real;
    float dt = -logf(u01_open0_f(u)) / rate;
    double t1 = t + (double)dt;
    return t1 < p.max_time ? t1 : p.max_time;
}

// Records the end of a trajectory: final-state histogram, fixed-point buffer, optional per
// trajectory records. Called by one lane (thread path) or with lane 0 as leader (warp path);
// `words` points at the W state words (registers or shared memory).
__device__ __forceinline__ void record_end_scalar(const SimParams& p, unsigned long long j, unsigned char status,
                                                  double t, unsigned trans, unsigned out_idx) {
    if (status == TRAJ_FINISHED || status == TRAJ_FIXED_POINT) atomicAdd(p.final_hist + out_idx, 1u);
    if (p.traj_time) p.traj_time[j] = t;
    if (p.traj_transitions) p.traj_transitions[j] = trans;
    if (p.traj_status) p.traj_status[j] = status;
}

// ---------------------------------------------------------------------------------------------
// Thread-per-trajectory kernel over a model policy M with compile-time word count M::W:
//   M::eval(p, s, act, rout, cout) -> total fixed-point rate; fills the active bits
//   M::pick(p, s, act, r)          -> first node whose prefix exceeds r
//   M::out_index(p, s)             -> output state index
// Lanes take new trajectories from a shared work counter, one warp-aggregated atomic per refill,
// so a warp stays full while its trajectories end at different times.

template <class M>
__device__ __forceinline__ void thread_init_state(const SimParams& p, unsigned long long traj, unsigned (&s)[M::W]) {
#pragma unroll
    for (int w = 0; w < M::W; ++w) s[w] = 0u;
    const int n = p.n;
    for (int b = 0; 4 * b < n; ++b) {
        u32x4 d = philox_init(p.seed, traj, (unsigned)b);
        unsigned v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int i = 4 * b + c;
            if (i < n && (v[c] >> 8) < __ldg(p.istate_thr + i)) {
#pragma unroll
                for (int w = 0; w < M::W; ++w)
                    if (w == (i >> 5)) s[w] |= 1u << (i & 31);
            }
        }
    }
}

template <class M>
__device__ void sim_thread_body(const SimParams& p) {
    constexpr int W = M::W;
    const unsigned lane = threadIdx.x & 31u;
    unsigned s[W], act[W];
    unsigned long long j = 0, step = 0;
    double t = 0.0;
    unsigned trans = 0;
    bool have = false, done = false;
    WindowAcc acc;
    unsigned long long c_trans = 0, c_steps = 0;
    unsigned c_fin = 0, c_fix = 0, c_lim = 0, c_err = 0;

    for (;;) {
        unsigned need = __ballot_sync(MBG_FULL, !have && !done);
        if (need) {
            unsigned long long base = 0;
            int leader = __ffs(need) - 1;
            if ((int)lane == leader) base = atomicAdd(p.counters + CNT_WORK, (unsigned long long)__popc(need));
            base = __shfl_sync(MBG_FULL, base, leader);
            if (!have && !done) {
                j = base + __popc(need & ((1u << lane) - 1u));
                if (j < p.n_traj) {
                    thread_init_state<M>(p, p.traj_base + j, s);
                    have = true;
                    t = 0.0;
                    step = 0;
                    trans = 0;
                    win_begin(acc, p, M::out_index(p, s));
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(MBG_FULL, done)) break;
        if (!have) continue;

        unsigned long long rout;
        float cout;
        const unsigned long long total = M::eval(p, s, act, rout, cout);
        const unsigned so = M::out_index(p, s);
        unsigned char status = TRAJ_CONTINUE;
        if (total == 0ull) {
            if (p.discrete) win_discrete(p, step, so, 0.f, true);
            else win_slice(acc, p, t, p.max_time, so, 0.f, true);
            t = p.max_time;
            status = TRAJ_FIXED_POINT;
        } else if (step >= p.max_steps) {
            status = TRAJ_STEP_LIMIT;
        } else {
            const float h = entropy_from_sums(rout, cout, p.to_real);
            const u32x4 d = philox_step(p.seed, p.traj_base + j, step);
            const double t1 = next_time(p, t, step, d.x, total);
            if (p.discrete) win_discrete(p, step, so, h, true);
            else win_slice(acc, p, t, t1, so, h, true);
            ++step;
            if (t1 >= p.max_time) {
                t = p.max_time;
                status = TRAJ_FINISHED;
            } else {
                const unsigned long long r = pick_target(d.y, d.z, total);
                const int k = M::pick(p, s, act, r);
                if (k < 0 || k >= p.n) {
                    status = TRAJ_ERROR;
                    atomicOr(p.error_flag, (unsigned)DEV_ERR_PICK);
                } else {
#pragma unroll
                    for (int w = 0; w < W; ++w)
                        if (w == (k >> 5)) s[w] ^= 1u << (k & 31);
                    t = t1;
                    ++trans;
                }
            }
        }
        if (status != TRAJ_CONTINUE) {
            if (!p.discrete && status != TRAJ_ERROR) win_end(acc, p, t, true);
            const unsigned char st = status;
            c_trans += trans;
            c_steps += step + (st == TRAJ_FIXED_POINT ? 1 : 0);
            c_fin += st == TRAJ_FINISHED;
            c_fix += st == TRAJ_FIXED_POINT;
            c_lim += st == TRAJ_STEP_LIMIT;
            c_err += st == TRAJ_ERROR;
            record_end_scalar(p, j, st, t, trans, M::out_index(p, s));
            if (p.traj_state) {
#pragma unroll
                for (int w = 0; w < W; ++w)
                    if (w < p.words) p.traj_state[j * p.words + w] = s[w];
            }
            if (st == TRAJ_FIXED_POINT) {
                unsigned slot = atomicAdd(p.fp_count, 1u);
                if (slot < p.fp_capacity) {
#pragma unroll
                    for (int w = 0; w < W; ++w)
                        if (w < p.words) p.fp_states[(unsigned long long)slot * p.words + w] = s[w];
                } else {
                    atomicOr(p.error_flag, (unsigned)DEV_ERR_FP_OVERFLOW);
                }
            }
            have = false;
        }
    }
    // counters: one atomic per warp and counter
    for (int o = 16; o > 0; o >>= 1) {
        c_trans += __shfl_xor_sync(MBG_FULL, c_trans, o);
        c_steps += __shfl_xor_sync(MBG_FULL, c_steps, o);
    }
    c_fin = __reduce_add_sync(MBG_FULL, c_fin);
    c_fix = __reduce_add_sync(MBG_FULL, c_fix);
    c_lim = __reduce_add_sync(MBG_FULL, c_lim);
    c_err = __reduce_add_sync(MBG_FULL, c_err);
    if (lane == 0) {
        atomicAdd(p.counters + CNT_TRANSITIONS, c_trans);
        atomicAdd(p.counters + CNT_STEPS, c_steps);
        atomicAdd(p.counters + CNT_FINISHED, (unsigned long long)c_fin);
        atomicAdd(p.counters + CNT_FIXED, (unsigned long long)c_fix);
        atomicAdd(p.counters + CNT_STEP_LIMIT, (unsigned long long)c_lim);
        atomicAdd(p.counters + CNT_ERROR, (unsigned long long)c_err);
    }
}

}  // namespace mbg
