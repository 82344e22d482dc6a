// Thread-per-trajectory kernel body over a model policy M with compile-time word count M::W:
//   M::eval(p, s, act, rout, cout) -> total fixed-point rate; fills the active bits
//   M::pick(p, s, act, r)          -> first node whose prefix exceeds r
//   M::out_index(p, s)             -> output state index
// The policy is generated per model and compiled by NVRTC (codegen.cpp). Lanes take new
// trajectories from a shared work counter, one warp-aggregated atomic per refill, so a warp stays
// full while its trajectories end at different times. Includes nothing (NVRTC program part).
#pragma once

namespace mbg {

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
    unsigned long long j = 0, step = 0, t = 0;
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
                    t = 0;
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
            else win_slice(acc, p, t, p.max_time_fx, so, 0.f, true);
            t = p.max_time_fx;
            status = TRAJ_FIXED_POINT;
        } else if (step >= p.max_steps) {
            status = TRAJ_STEP_LIMIT;
        } else {
            const float h = entropy_from_sums(rout, cout, p.to_real);
            const u32x4 d = philox_step(p.seed, p.traj_base + j, step);
            const unsigned long long t1 = next_time(p, t, step, p.discrete ? 0.f : neg_log_u(d.x), total);
            if (p.discrete) win_discrete(p, step, so, h, true);
            else win_slice(acc, p, t, t1, so, h, true);
            ++step;
            if (t1 >= p.max_time_fx) {
                t = p.max_time_fx;
                status = TRAJ_FINISHED;
            } else if (p.redraw_period && step % p.redraw_period == 0ull) {
                t = t1;  // a reference segment ends: the holding time is drawn again, no flip
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
