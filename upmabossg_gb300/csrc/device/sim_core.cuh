// Device building blocks shared by the thread-per-trajectory kernels (NVRTC-compiled per model)
// and the warp-per-trajectory kernel. Includes nothing: sim_types.h and philox.h come first in
// both the nvcc and the NVRTC translation unit.
//
// Per-trajectory semantics restate src/jit_kernels/simulation.cu:77-164:
//   * a state with total rate 0 is a fixed point and holds until max_time (114-118);
//   * otherwise dt = -log(U) / total (FP32), the clock is clamped to max_time (129-131), and the
//     slice [t, t+dt] is credited to the state held before the flip (137-147);
//   * the trajectory ends when the clock reaches max_time (143);
//   * the flipped node is the first whose rate prefix passes the target (select_flip_bit, 9-21),
//     here with exact 64-bit fixed-point rates.
// The clock itself is an unsigned fixed-point number with p.time_bits fraction bits (the
// reference keeps it in FP32): every step adds the FP32 dt rounded to that grid, so the loop has
// no FP64 instruction, and window edges are exact multiples of the rounded tick.
// Window accumulation restates src/jit_kernels/window_average_small.cu:64-93: a slice is split at
// the window edges w*tick and each piece is added to bin [w][output state]; the transition
// entropy is added weighted by the piece length. Consecutive slices in the same (window, state)
// are merged before they are written, so one trajectory issues about one atomic per change of
// output state. Bins are 64-bit fixed point (2^-32 time units), which makes the result independent
// of the order of the atomics.
#pragma once

namespace mbg {

#define MBG_FULL 0xffffffffu

// round(x * 2^bits) for a finite x >= 0, saturating at 2^62; zero and denormals give 0.
__device__ __forceinline__ unsigned long long f32_to_fixed(float x, int bits) {
    const unsigned b = __float_as_uint(x);
    const int e = (int)((b >> 23) & 0xffu);
    if (e == 0) return 0ull;
    const unsigned long long m = (b & 0x7fffffu) | 0x800000u;  // x = m * 2^(e - 150)
    const int sh = e - 150 + bits;
    if (sh >= 0) return sh > 38 ? (1ull << 62) : (m << sh);
    if (sh < -25) return 0ull;
    return (m + (1ull << (-sh - 1))) >> (-sh);
}

// u64 to float without the 64-bit conversion instruction: two exact 32-bit halves.
__device__ __forceinline__ float u64_to_f32(unsigned long long v) {
    return (float)(unsigned)(v >> 32) * 4294967296.0f + (float)(unsigned)v;
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

// A clock interval in real time units.
__device__ __forceinline__ float fx_to_time(const SimParams& p, unsigned long long v) {
    return u64_to_f32(v) * pow2f(-p.time_bits);
}

// A clock interval in the 2^-32 units of the window sums.
__device__ __forceinline__ unsigned long long fx_to_bin(const SimParams& p, unsigned long long v) {
    const int sh = p.time_bits - 32;
    return sh > 0 ? (v + (1ull << (sh - 1))) >> sh : v;
}

struct WindowAcc {
    int w;                     // current window
    unsigned long long wend;   // end of window w (clock units)
    unsigned long long run_t0; // start of the current run of one output state inside window w
    unsigned run_s;            // output state of the run
    float th;                  // sum of TH x length inside window w (time units)
};

__device__ __forceinline__ void win_begin(WindowAcc& a, const SimParams& p, unsigned s) {
    a.w = 0;
    a.wend = p.tick_fx;
    a.run_t0 = 0ull;
    a.run_s = s;
    a.th = 0.f;
}

// Window sums go to the dense table or to the hash table; which one is fixed when a kernel is
// compiled (MBG_WINDOW_HASH 0 or 1): the dense kernels carry no trace of the hash path, whose
// probe loop, inlined at every flush, cost the 5000-node warp kernel 6% when both were compiled in
// behind a run-time branch. The host launches the variant that matches the run's table.
#ifndef MBG_WINDOW_HASH
#define MBG_WINDOW_HASH 0
#endif

// Probes one insertion into the window hash table may take before it gives up (the host then
// re-runs with a larger table). The host keeps the table at most half full.
#define MBG_WINDOW_PROBES 512u

// Slot of `key` (bin + 1) in a table of 2^bits slots: the top bits of its Fibonacci product.
__device__ __forceinline__ unsigned long long win_hash(unsigned long long key, int bits) {
    return (key * 0x9E3779B97F4A7C15ull) >> (64 - bits);
}

// Adds v to the window sum of bin (window w, output state s): one atomic on the dense table, or,
// in the hash kernels, a claim-or-match of the bin's slot followed by an atomic add on its sum.
// The sums are integers, so the result depends neither on the order of the additions nor on which
// trajectory claimed a slot. A slot's key, once set, never changes during a run, so a cached load
// that finds the key is exact and skips the CAS; a load that finds the slot empty (possibly stale)
// falls through to the CAS, which returns the truth.
__device__ __forceinline__ void bin_add(const SimParams& p, int w, unsigned s, unsigned long long v) {
    const unsigned long long bin = ((unsigned long long)w << p.n_out) | s;
#if MBG_WINDOW_HASH
    const unsigned long long key = bin + 1ull;
    const unsigned long long mask = (1ull << p.hash_bits) - 1ull;
    unsigned long long h = win_hash(key, p.hash_bits);
    for (unsigned probe = 0; probe < MBG_WINDOW_PROBES; ++probe) {
        unsigned long long* slot = p.hslots + 2 * h;
        unsigned long long cur = __ldca(slot);
        if (cur == 0ull) {
            cur = atomicCAS(slot, 0ull, key);
            if (cur == 0ull) {
                atomicAdd(slot + 1, v);
                atomicAdd(p.counters + CNT_WIN_ENTRIES, 1ull);
                return;
            }
        }
        if (cur == key) {
            atomicAdd(slot + 1, v);
            return;
        }
        h = (h + 1ull) & mask;
        // once any insertion has overflowed the run is repeated anyway: stop probing early
        if ((probe & 15u) == 15u && (*(volatile const unsigned*)p.error_flag & (unsigned)DEV_ERR_WINDOW_TABLE)) return;
    }
    atomicOr(p.error_flag, (unsigned)DEV_ERR_WINDOW_TABLE);
#else
    atomicAdd(p.hist + bin, v);
#endif
}

__device__ __forceinline__ void win_flush_run(WindowAcc& a, const SimParams& p, unsigned long long t_end,
                                              bool leader) {
    if (leader && t_end > a.run_t0) bin_add(p, a.w, a.run_s, fx_to_bin(p, t_end - a.run_t0));
}

__device__ __forceinline__ void win_flush_th(WindowAcc& a, const SimParams& p, bool leader) {
    if (leader && a.th != 0.f) atomicAdd(p.th_hist + a.w, f32_to_fixed(a.th, 32));
    a.th = 0.f;
}

// Continuous time: the output state s with entropy h was held over [t0, t1].
__device__ __forceinline__ void win_slice(WindowAcc& a, const SimParams& p, unsigned long long t0,
                                          unsigned long long t1, unsigned s, float h, bool leader) {
    if (s != a.run_s) {
        win_flush_run(a, p, t0, leader);
        a.run_s = s;
        a.run_t0 = t0;
    }
    while (t1 > a.wend && a.w + 1 < p.windows) {
        a.th += h * fx_to_time(p, a.wend - t0);
        win_flush_run(a, p, a.wend, leader);
        win_flush_th(a, p, leader);
        t0 = a.wend;
        a.run_t0 = t0;
        a.w += 1;
        a.wend = (unsigned long long)(a.w + 1) * p.tick_fx;
    }
    a.th += h * fx_to_time(p, t1 - t0);
}

__device__ __forceinline__ void win_end(WindowAcc& a, const SimParams& p, unsigned long long t_end, bool leader) {
    win_flush_run(a, p, t_end, leader);
    win_flush_th(a, p, leader);
}

// Discrete time (window_average_small.cu:101-136): one count per recorded step, in the window of
// the step's start time, which is step * tick.
__device__ __forceinline__ void win_discrete(const SimParams& p, unsigned long long step, unsigned s, float h,
                                             bool leader) {
    int w = step < (unsigned long long)p.windows ? (int)step : p.windows - 1;
    if (leader) {
        bin_add(p, w, s, 1ull);
        if (h != 0.f) atomicAdd(p.th_hist + w, f32_to_fixed(h, 32));
    }
}

// Transition entropy from the summed output rates (fixed point) and sum r*log2(r) (real units):
// -sum p log2 p = log2 R - (sum r log2 r) / R.
__device__ __forceinline__ float entropy_from_sums(unsigned long long rout, float cout, float to_real) {
    if (rout == 0ull) return 0.f;
    const float R = u64_to_f32(rout) * to_real;
    const float h = __log2f(R) - __fdividef(cout, R);
    return h > 0.f ? h : 0.f;
}

// -ln(U) for the dt draw u (one Philox word).
__device__ __forceinline__ float neg_log_u(unsigned u) { return -logf(u01_open0_f(u)); }

// End of the step that starts at clock t: t + dt (continuous, dt = nlog / total) or the next tick
// (discrete), clamped to max_time.
__device__ __forceinline__ unsigned long long next_time(const SimParams& p, unsigned long long t,
                                                        unsigned long long step, float nlog,
                                                        unsigned long long total) {
    if (p.discrete) {
        return (step + 1 >= (unsigned long long)p.windows) ? p.max_time_fx
                                                           : (unsigned long long)(step + 1) * p.tick_fx;
    }
    const float rate = u64_to_f32(total) * p.to_real;
    const unsigned long long t1 = t + f32_to_fixed(__fdividef(nlog, rate), p.time_bits);
    return t1 < p.max_time_fx ? t1 : p.max_time_fx;
}

__device__ __forceinline__ double fx_to_double(const SimParams& p, unsigned long long t) {
    return (double)t * (double)pow2f(-p.time_bits);
}

// Records the end of a trajectory: final-state histogram and the optional per-trajectory
// records. Called by one lane (thread path) or by lane 0 (warp path).
__device__ __forceinline__ void record_end_scalar(const SimParams& p, unsigned long long j, unsigned char status,
                                                  unsigned long long t, unsigned trans, unsigned out_idx) {
    if (status == TRAJ_FINISHED || status == TRAJ_FIXED_POINT) atomicAdd(p.final_hist + out_idx, 1u);
    if (p.traj_time) p.traj_time[j] = fx_to_double(p, t);
    if (p.traj_transitions) p.traj_transitions[j] = trans;
    if (p.traj_status) p.traj_status[j] = status;
}

}  // namespace mbg
