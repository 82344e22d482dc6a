// One trajectory per lane, table-driven, with the state in shared memory and every rate kept
// up to date incrementally (the "lane" layout).
//
// The reference re-evaluates all N rates and scans them on every step
// (src/jit_kernels/simulation.cu:9-21 and 77-164 with the generated compute_transition_rates of
// src/generator.cpp:124-144). Here a lane keeps, for its trajectory:
//   st[W]    state words,
//   act[W]   active words (bit i: node i's rate is non-zero),
//   gsum[G]  exact 64-bit fixed-point rate sum of each 32-node group (G = W),
//   gact[GW] bit g: gsum[g] != 0,
// in shared memory, in rows of blockDim.x entries (entry [row][thread]), so that the 32 lanes of a
// warp always touch 32 distinct banks whatever rows they read. A step walks the non-empty groups in
// node order, then the active nodes of the chosen group, which is the reference's first-prefix
// pick restricted to the nodes that can contribute; a flip of node k re-evaluates only the nodes
// whose rate reads k (the dependency CSR) and patches act, gsum, gact and the total. Every lane
// runs its own trajectory, so the per-step work is not spread over a warp; a new trajectory is set
// up by the whole warp at once (one node per lane), because that pass is O(N).
// Includes nothing: sim_types.h, philox.h, sim_core.cuh and sim_warp.cuh come first.
#pragma once

namespace mbg {

__host__ __device__ __forceinline__ int lane_groups(int n) { return (n + 31) >> 5; }
__host__ __device__ __forceinline__ int lane_gwords(int n) { return (lane_groups(n) + 31) >> 5; }
// Shared-memory bytes per thread: group sums, the rate-change slot, state, active and
// non-empty-group words, the output-touched slot.
__host__ __device__ __forceinline__ unsigned lane_smem_bytes(int n) {
    const int G = lane_groups(n);
    return (unsigned)(8 * (G + 1) + 4 * (2 * G + lane_gwords(n) + 1));
}

struct LaneSmem {
    unsigned long long* gsum;    // [G][T]
    unsigned long long* tdelta;  // [T]: rate change of the owner's total during a cooperative update
    unsigned* st;                // [G][T]
    unsigned* act;               // [G][T]
    unsigned* gact;              // [GW][T]
    unsigned* touched;           // [T]: an output node's rate changed
};

__device__ __forceinline__ LaneSmem lane_smem_at(unsigned char* base, int n, int T) {
    const int G = lane_groups(n);
    LaneSmem m;
    m.gsum = reinterpret_cast<unsigned long long*>(base);
    m.tdelta = m.gsum + (size_t)G * T;
    m.st = reinterpret_cast<unsigned*>(m.tdelta + T);
    m.act = m.st + (size_t)G * T;
    m.gact = m.act + (size_t)G * T;
    m.touched = m.gact + (size_t)lane_gwords(n) * T;
    return m;
}

// Bit i of a per-thread bit vector stored as rows of T words (`col` points at the thread's entry
// of row 0).
__device__ __forceinline__ unsigned col_bit(const unsigned* col, int T, int i) {
    return (col[(i >> 5) * T] >> (i & 31)) & 1u;
}

// Regulator index of node i (k regulators) in the state column st.
__device__ __forceinline__ unsigned lane_gather(const SimParams& p, int i, int k, const unsigned* st, int T) {
    unsigned idx = 0u;
    const unsigned short* inl = p.nodes[i].r;
    const int kin = k < kInlineRegs ? k : kInlineRegs;
    for (int j = 0; j < kin; ++j) idx |= col_bit(st, T, __ldg(inl + j)) << j;
    if (k > kInlineRegs) {
        const unsigned short* far = p.regs + __ldg(&p.nodes[i].reg_off);
        for (int j = kInlineRegs; j < k; ++j) idx |= col_bit(st, T, __ldg(far + j)) << j;
    }
    return idx;
}

// Regulator index of a node with k <= 4 regulators packed as r01 = r0 | r1 << 16, r23 likewise.
__device__ __forceinline__ unsigned lane_idx4(const unsigned* st, int T, int k, unsigned r01, unsigned r23) {
    unsigned idx = 0u;
    if (k > 0) idx |= col_bit(st, T, (int)(r01 & 0xffffu));
    if (k > 1) idx |= col_bit(st, T, (int)(r01 >> 16)) << 1;
    if (k > 2) idx |= col_bit(st, T, (int)(r23 & 0xffffu)) << 2;
    if (k > 3) idx |= col_bit(st, T, (int)(r23 >> 16)) << 3;
    return idx;
}

// Current rate of node i from its active bit (BINARY) or its table (PALETTE).
__device__ __forceinline__ unsigned long long lane_rate(const SimParams& p, int i, const unsigned* st,
                                                        const unsigned* act, int T) {
    const unsigned self = col_bit(st, T, i);
    if (p.has_palette && (__ldg(&p.lnodes[i].flags) & kLanePalette)) {
        const NodeHead h = load_head(p, i);
        return palette_rate(p, h, self, lane_gather(p, i, h.k, st, T));
    }
    if (!col_bit(act, T, i)) return 0ull;
    return __ldg(&p.lnodes[i].up + self);
}

// Output-state index: bit q = state of output node q.
__device__ __forceinline__ unsigned lane_out_index(const SimParams& p, const unsigned* st, int T) {
    unsigned so = 0u;
    for (int q = 0; q < p.n_out; ++q) so |= col_bit(st, T, __ldg(p.out_nodes + q)) << q;
    return so;
}

// Transition entropy over the output nodes (generator.cpp:146-175) from one pass:
// -sum p log2 p = log2 R - (sum r log2 r) / R.
__device__ __forceinline__ float lane_entropy(const SimParams& p, const unsigned* st, const unsigned* act, int T) {
    unsigned long long R = 0ull;
    float c = 0.f;
    for (int q = 0; q < p.n_out; ++q) {
        const unsigned long long r = lane_rate(p, __ldg(p.out_nodes + q), st, act, T);
        if (r) {
            R += r;
            const float rr = u64_to_f32(r) * p.to_real;
            c += rr * __log2f(rr);
        }
    }
    return entropy_from_sums(R, c, p.to_real);
}

// The whole warp sets up the trajectory `traj` in column `c` (state, active bits, group sums,
// non-empty-group bits); returns the total rate on every lane.
__device__ __forceinline__ unsigned long long lane_coop_init(const SimParams& p, const LaneSmem& m, int T, int c,
                                                             unsigned long long traj, unsigned lane) {
    const int n = p.n, G = lane_groups(n), GW = lane_gwords(n);
    unsigned* st = m.st + c;
    // state word w from Philox blocks 8w .. 8w+7 (4 nodes each), as the other layouts do
    for (int w = (int)lane; w < G; w += 32) {
        unsigned word = 0u;
        for (int b = 0; b < 8; ++b) {
            const int blk = w * 8 + b;
            if (4 * blk >= n) break;
            const u32x4 d = philox_init(p.seed, traj, (unsigned)blk);
            const unsigned v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int i = 4 * blk + q;
                if (i < n && (v[q] >> 8) < __ldg(p.istate_thr + i)) word |= 1u << (i & 31);
            }
        }
        st[w * T] = word;
    }
    __syncwarp();
    unsigned long long total = 0ull;
    unsigned gbits = 0u;  // lane q collects bits of gact word q
    for (int g = 0; g < G; ++g) {
        const int i = g * 32 + (int)lane;
        unsigned long long v = 0ull;
        if (i < n) {
            const uint4* rec = reinterpret_cast<const uint4*>(p.lnodes + i);
            const uint4 ra = __ldg(rec), rb = __ldg(rec + 1);
            const unsigned self = col_bit(st, T, i);
            if ((rb.w >> 16) == 0u) {
                const unsigned idx = lane_idx4(st, T, (int)(rb.w & 0xffffu), rb.y, rb.z);
                const int k = (int)(rb.w & 0xffffu);
                if ((rb.x >> ((self << k) | idx)) & 1u)
                    v = self ? (((unsigned long long)ra.w << 32) | ra.z) : (((unsigned long long)ra.y << 32) | ra.x);
            } else {
                const NodeHead h = load_head(p, i);
                v = rate_at(p, i, h, self, lane_gather(p, i, h.k, st, T));
            }
        }
        const unsigned a = __ballot_sync(MBG_FULL, v != 0ull);
        const unsigned long long s = warp_sum_u64(v);
        if (lane == 0u) {
            m.act[g * T + c] = a;
            m.gsum[(size_t)g * T + c] = s;
        }
        if (s != 0ull && (int)lane == (g >> 5)) gbits |= 1u << (g & 31);
        total += s;
    }
    if ((int)lane < GW) m.gact[lane * T + c] = gbits;
    if (lane == 0u) {
        m.tdelta[c] = 0ull;
        m.touched[c] = 0u;
    }
    __syncwarp();
    return total;
}

// First node whose inclusive rate prefix exceeds r (r < total), or -1.
__device__ __forceinline__ int lane_pick(const SimParams& p, const unsigned* st, const unsigned* act,
                                         const unsigned long long* gs, const unsigned* ga, int T, int GW,
                                         unsigned long long r) {
    int g = -1;
    for (int gw = 0; gw < GW && g < 0; ++gw) {
        unsigned bits = ga[gw * T];
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1u;
            const int gg = gw * 32 + b;
            const unsigned long long s = gs[(size_t)gg * T];
            if (r < s) {
                g = gg;
                break;
            }
            r -= s;
        }
    }
    if (g < 0) return -1;
    unsigned aw = act[g * T];
    const unsigned sw = st[g * T];
    while (aw) {
        const int b = __ffs(aw) - 1;
        aw &= aw - 1u;
        const int i = g * 32 + b;
        const unsigned long long v =
            p.has_palette ? lane_rate(p, i, st, act, T) : __ldg(&p.lnodes[i].up + ((sw >> b) & 1u));
        if (r < v) return i;
        r -= v;
    }
    return -1;
}

// Re-evaluates reader dn of a node that just flipped, in the trajectory whose entries start at
// `col`: dependency entry e = (dn << 16) | (k_dn << 8) | pos (pos 0xFF: dn itself flipped). Patches
// act, gsum and gact (with shared-memory atomics when several lanes may patch the same
// trajectory), returns the rate change and sets `out` when dn is an output node whose rate changed.
template <bool ATOMIC>
__device__ __forceinline__ unsigned long long lane_reader(const SimParams& p, unsigned e, const LaneSmem& m, int T,
                                                          int col, bool& out) {
    const int dn = (int)(e >> 16);
    const int kd = (int)((e >> 8) & 0xffu);
    const unsigned pos = e & 0xffu;
    const unsigned* st = m.st + col;
    const unsigned self = col_bit(st, T, dn);
    const unsigned self_old = pos == 0xffu ? self ^ 1u : self;
    const uint4* rec = reinterpret_cast<const uint4*>(p.lnodes + dn);
    const uint4 ra = __ldg(rec), rb = __ldg(rec + 1);
    const unsigned flags = rb.w >> 16;
    unsigned long long r_new, r_old;
    unsigned a_new, a_old;
    if (!(flags & kLanePalette)) {
        if (flags == 0u) {
            // up to 4 regulators and their table in the record itself
            a_new = (rb.x >> ((self << kd) | lane_idx4(st, T, kd, rb.y, rb.z))) & 1u;
        } else {
            a_new = table_bit(p, dn, kd, self, lane_gather(p, dn, kd, st, T));
        }
        a_old = col_bit(m.act + col, T, dn);
        if (a_new == a_old && pos != 0xffu) return 0ull;  // a reader whose rate did not change
        const unsigned long long up = ((unsigned long long)ra.y << 32) | ra.x;
        const unsigned long long down = ((unsigned long long)ra.w << 32) | ra.z;
        r_new = a_new ? (self ? down : up) : 0ull;
        r_old = a_old ? (self_old ? down : up) : 0ull;
    } else {
        const NodeHead h = load_head(p, dn);
        const unsigned idx = lane_gather(p, dn, kd, st, T);
        const unsigned idx_old = pos == 0xffu ? idx : idx ^ (1u << pos);
        r_new = palette_rate(p, h, self, idx);
        r_old = palette_rate(p, h, self_old, idx_old);
        a_new = r_new != 0ull;
        a_old = r_old != 0ull;
    }
    const int g = dn >> 5;
    unsigned* aw = m.act + (size_t)g * T + col;
    unsigned long long* gw = m.gsum + (size_t)g * T + col;
    unsigned* gaw = m.gact + (size_t)(g >> 5) * T + col;
    if (a_new != a_old) {
        if (ATOMIC) atomicXor(aw, 1u << (dn & 31));
        else *aw ^= 1u << (dn & 31);
    }
    const unsigned long long delta = r_new - r_old;
    if (delta != 0ull) {
        // the non-empty bit follows every change of the sum; under atomics each update sees a
        // consistent predecessor, so the toggles compose to (final sum != 0)
        unsigned long long s_old;
        if (ATOMIC) {
            s_old = atomicAdd(gw, delta);
        } else {
            s_old = *gw;
            *gw = s_old + delta;
        }
        if ((s_old == 0ull) != (s_old + delta == 0ull)) {
            if (ATOMIC) atomicXor(gaw, 1u << (g & 31));
            else *gaw ^= 1u << (g & 31);
        }
        out |= __ldg(p.out_pos + dn) >= 0;
    }
    return delta;
}

// After node k flipped in this lane's trajectory: re-evaluates every node whose rate reads k (and
// k itself) in turn. Returns whether an output node's rate changed.
__device__ __forceinline__ bool lane_update(const SimParams& p, int k, const LaneSmem& m, int T, int col,
                                            unsigned long long& total) {
    const int d0 = (int)__ldg(p.dep_off + k), d1 = (int)__ldg(p.dep_off + k + 1);
    bool out = false;
    for (int q = d0; q < d1; ++q) total += lane_reader<false>(p, __ldg(p.deps + q), m, T, col, out);
    return out;
}

// Warp-cooperative form of lane_update for every lane at once (k < 0: nothing flipped): the
// reader lists of the 32 flipped nodes are concatenated and dealt out one entry per lane, so a
// step costs ceil(total length / 32) rounds instead of the longest list. Entries of one trajectory
// patch its shared-memory rows with atomics and add their rate changes to its tdelta slot.
__device__ __forceinline__ void lane_coop_update(const SimParams& p, const LaneSmem& m, int T, int wbase,
                                                 unsigned lane, int k) {
    int d0 = 0, c = 0;
    if (k >= 0) {
        d0 = (int)__ldg(p.dep_off + k);
        c = (int)__ldg(p.dep_off + k + 1) - d0;
    }
    int inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(MBG_FULL, inc, o);
        if ((int)lane >= o) inc += v;
    }
    const int C = __shfl_sync(MBG_FULL, inc, 31);
    const int ex = inc - c;
    __syncwarp();  // every lane's flip is visible
    for (int base = 0; base < C; base += 32) {
        const int q = base + (int)lane;
        // owner: the first lane whose inclusive count exceeds q
        int o = 0;
#pragma unroll
        for (int s = 16; s >= 1; s >>= 1) {
            const int v = __shfl_sync(MBG_FULL, inc, o + s - 1);
            if (v <= q) o += s;
        }
        const int o_ex = __shfl_sync(MBG_FULL, ex, o);
        const int o_d0 = __shfl_sync(MBG_FULL, d0, o);
        if (q < C) {
            const int col = wbase + o;
            bool out = false;
            const unsigned long long delta = lane_reader<true>(p, __ldg(p.deps + o_d0 + (q - o_ex)), m, T, col, out);
            if (delta != 0ull) atomicAdd(m.tdelta + col, delta);
            if (out) atomicOr(m.touched + col, 1u);
        }
    }
    __syncwarp();
}

template <bool COOP>
__device__ void sim_lane_body(const SimParams& p, unsigned char* smem) {
    const int T = (int)blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const int wbase = (int)(threadIdx.x & ~31u);
    const int GW = lane_gwords(p.n);
    const LaneSmem m = lane_smem_at(smem, p.n, T);
    const int col = (int)threadIdx.x;
    unsigned* st = m.st + col;
    const unsigned* act = m.act + col;
    const unsigned long long* gs = m.gsum + col;
    const unsigned* ga = m.gact + col;

    unsigned long long j = 0, step = 0, t = 0, total = 0;
    unsigned trans = 0, so = 0;
    float h = 0.f;
    bool have = false, done = false;
    WindowAcc acc;
    unsigned long long c_trans = 0, c_steps = 0;
    unsigned c_fin = 0, c_fix = 0, c_lim = 0, c_err = 0;

    for (;;) {
        const unsigned need = __ballot_sync(MBG_FULL, !have && !done);
        if (need) {
            unsigned long long base = 0;
            const int leader = __ffs(need) - 1;
            if ((int)lane == leader) base = atomicAdd(p.counters + CNT_WORK, (unsigned long long)__popc(need));
            base = __shfl_sync(MBG_FULL, base, leader);
            bool start = false;
            if (!have && !done) {
                j = base + __popc(need & ((1u << lane) - 1u));
                if (j < p.n_traj) start = true;
                else done = true;
            }
            unsigned init = __ballot_sync(MBG_FULL, start);
            while (init) {
                const int L = __ffs(init) - 1;
                init &= init - 1u;
                const unsigned long long jl = __shfl_sync(MBG_FULL, j, L);
                const unsigned long long tot = lane_coop_init(p, m, T, wbase + L, p.traj_base + jl, lane);
                if ((int)lane == L) total = tot;
            }
            if (start) {
                have = true;
                t = 0;
                step = 0;
                trans = 0;
                so = lane_out_index(p, st, T);
                h = lane_entropy(p, st, act, T);
                win_begin(acc, p, so);
            }
        }
        if (__all_sync(MBG_FULL, done)) break;
        if (!COOP && !have) continue;

        unsigned char status = TRAJ_CONTINUE;
        int k = -1;
        unsigned long long t1 = 0;
        if (have) {
            if (total == 0ull) {
                if (p.discrete) win_discrete(p, step, so, 0.f, true);
                else win_slice(acc, p, t, p.max_time_fx, so, 0.f, true);
                t = p.max_time_fx;
                status = TRAJ_FIXED_POINT;
            } else if (step >= p.max_steps) {
                status = TRAJ_STEP_LIMIT;
            } else {
                const u32x4 d = philox_step(p.seed, p.traj_base + j, step);
                t1 = next_time(p, t, step, p.discrete ? 0.f : neg_log_u(d.x), total);
                if (p.discrete) win_discrete(p, step, so, h, true);
                else win_slice(acc, p, t, t1, so, h, true);
                ++step;
                if (t1 >= p.max_time_fx) {
                    t = p.max_time_fx;
                    status = TRAJ_FINISHED;
                } else {
                    k = lane_pick(p, st, act, gs, ga, T, GW, pick_target(d.y, d.z, total));
                    if (k < 0 || k >= p.n) {
                        k = -1;
                        status = TRAJ_ERROR;
                        atomicOr(p.error_flag, (unsigned)DEV_ERR_PICK);
                    } else {
                        st[(k >> 5) * T] ^= 1u << (k & 31);
                        if (!COOP && lane_update(p, k, m, T, col, total)) h = lane_entropy(p, st, act, T);
                    }
                }
            }
        }
        if (COOP) {
            lane_coop_update(p, m, T, wbase, lane, k);
            if (k >= 0) {
                total += m.tdelta[col];
                m.tdelta[col] = 0ull;
                if (m.touched[col]) {
                    m.touched[col] = 0u;
                    h = lane_entropy(p, st, act, T);
                }
            }
        }
        if (k >= 0) {
            const short op = __ldg(p.out_pos + k);
            if (op >= 0) so ^= 1u << op;
            t = t1;
            ++trans;
        }
        if (status != TRAJ_CONTINUE) {
            if (!p.discrete && status != TRAJ_ERROR) win_end(acc, p, t, true);
            c_trans += trans;
            c_steps += step + (status == TRAJ_FIXED_POINT ? 1 : 0);
            c_fin += status == TRAJ_FINISHED;
            c_fix += status == TRAJ_FIXED_POINT;
            c_lim += status == TRAJ_STEP_LIMIT;
            c_err += status == TRAJ_ERROR;
            record_end_scalar(p, j, status, t, trans, so);
            if (p.traj_state)
                for (int w = 0; w < p.words; ++w) p.traj_state[j * p.words + w] = st[w * T];
            if (status == TRAJ_FIXED_POINT) {
                const unsigned slot = atomicAdd(p.fp_count, 1u);
                if (slot < p.fp_capacity) {
                    for (int w = 0; w < p.words; ++w) p.fp_states[(unsigned long long)slot * p.words + w] = st[w * T];
                } else {
                    atomicOr(p.error_flag, (unsigned)DEV_ERR_FP_OVERFLOW);
                }
            }
            have = false;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        c_trans += __shfl_xor_sync(MBG_FULL, c_trans, o);
        c_steps += __shfl_xor_sync(MBG_FULL, c_steps, o);
    }
    c_fin = __reduce_add_sync(MBG_FULL, c_fin);
    c_fix = __reduce_add_sync(MBG_FULL, c_fix);
    c_lim = __reduce_add_sync(MBG_FULL, c_lim);
    c_err = __reduce_add_sync(MBG_FULL, c_err);
    if (lane == 0u) {
        atomicAdd(p.counters + CNT_TRANSITIONS, c_trans);
        atomicAdd(p.counters + CNT_STEPS, c_steps);
        atomicAdd(p.counters + CNT_FINISHED, (unsigned long long)c_fin);
        atomicAdd(p.counters + CNT_FIXED, (unsigned long long)c_fix);
        atomicAdd(p.counters + CNT_STEP_LIMIT, (unsigned long long)c_lim);
        atomicAdd(p.counters + CNT_ERROR, (unsigned long long)c_err);
    }
}

}  // namespace mbg
