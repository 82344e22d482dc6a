// One trajectory per lane, table-driven, with the state in shared memory and every rate kept
// up to date incrementally (the "lane" layout).
//
// The reference re-evaluates all N rates and scans them on every step
// (src/jit_kernels/simulation.cu:9-21 and 77-164 with the generated compute_transition_rates of
// src/generator.cpp:124-144). Here a lane keeps, for its trajectory:
//   fen[G]  a Fenwick tree over the exact 64-bit fixed-point rate sums of the 32-node groups
//           (G = W): entry i (1-based) holds the sum of groups (i - lowbit(i), i],
//   st[W]   state words,
//   act[W]  active words (bit i: node i's rate is non-zero),
// in shared memory, in rows of blockDim.x entries (entry [row][thread]), so that the 32 lanes of a
// warp always touch 32 distinct banks whatever rows they read. A step descends the tree to the
// group holding the target (log2 G loads, the same count on every lane), then walks the active
// nodes of that group in node order: the reference's first-prefix pick, exactly. A flip of node k
// re-evaluates only the nodes whose rate reads k (the dependency CSR) and adds each rate change
// along its group's tree path. A new trajectory is set up by the whole warp at once (one node per
// lane), because that pass is O(N).
// Includes nothing: sim_types.h, philox.h, sim_core.cuh and sim_warp.cuh come first.
#pragma once

namespace mbg {

__host__ __device__ __forceinline__ int lane_groups(int n) { return (n + 31) >> 5; }
// Shared-memory bytes per thread (plus lane_block_extra per block).
__host__ __device__ __forceinline__ unsigned lane_smem_bytes(int n) { return 16u * (unsigned)lane_groups(n); }
// Per block: one word per warp (lanes whose output-node rates changed in a cooperative update).
__host__ __device__ __forceinline__ unsigned lane_block_extra(int block) { return 4u * (unsigned)((block + 31) / 32); }

struct LaneSmem {
    unsigned long long* fen;  // [G][T]
    unsigned* st;             // [G][T]
    unsigned* act;            // [G][T]
    unsigned* wtouch;         // [T / 32]
};

__device__ __forceinline__ LaneSmem lane_smem_at(unsigned char* base, int n, int T) {
    const int G = lane_groups(n);
    LaneSmem m;
    m.fen = reinterpret_cast<unsigned long long*>(base);
    m.st = reinterpret_cast<unsigned*>(m.fen + (size_t)G * T);
    m.act = m.st + (size_t)G * T;
    m.wtouch = m.act + (size_t)G * T;
    return m;
}

// Bit i of a per-thread bit vector stored as rows of T words (`col` points at the thread's entry
// of row 0).
__device__ __forceinline__ unsigned col_bit(const unsigned* col, int T, int i) {
    return (col[(i >> 5) * T] >> (i & 31)) & 1u;
}

// Fenwick tree of one trajectory (`col` points at its entry of row 0; tree index i is row i-1).
__device__ __forceinline__ void fen_add(unsigned long long* col, int T, int G, int g, unsigned long long delta) {
    for (int i = g + 1; i <= G; i += i & -i) col[(size_t)(i - 1) * T] += delta;
}
__device__ __forceinline__ void fen_add_atomic(unsigned long long* col, int T, int G, int g,
                                               unsigned long long delta) {
    for (int i = g + 1; i <= G; i += i & -i) atomicAdd(col + (size_t)(i - 1) * T, delta);
}
// Group holding target r (r < total): the largest g with sum(groups < g) <= r; r becomes relative
// to that group. `top` is the largest power of two <= G.
__device__ __forceinline__ int fen_find(const unsigned long long* col, int T, int G, int top,
                                        unsigned long long& r) {
    int pos = 0;
    for (int step = top; step > 0; step >>= 1) {
        const int nxt = pos + step;
        if (nxt <= G) {
            const unsigned long long v = col[(size_t)(nxt - 1) * T];
            if (v <= r) {
                pos = nxt;
                r -= v;
            }
        }
    }
    return pos;
}
__device__ __forceinline__ unsigned long long fen_total(const unsigned long long* col, int T, int G) {
    unsigned long long s = 0ull;
    for (int i = G; i > 0; i -= i & -i) s += col[(size_t)(i - 1) * T];
    return s;
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

// Rate of node i in the state column st, evaluated from its tables.
__device__ __forceinline__ unsigned long long lane_eval(const SimParams& p, int i, const unsigned* st, int T) {
    const uint4* rec = reinterpret_cast<const uint4*>(p.lnodes + i);
    const uint4 ra = __ldg(rec), rb = __ldg(rec + 1);
    const unsigned self = col_bit(st, T, i);
    if ((rb.w >> 16) == 0u) {
        const int k = (int)(rb.w & 0xffffu);
        if (!((rb.x >> ((self << k) | lane_idx4(st, T, k, rb.y, rb.z))) & 1u)) return 0ull;
        return self ? (((unsigned long long)ra.w << 32) | ra.z) : (((unsigned long long)ra.y << 32) | ra.x);
    }
    const NodeHead h = load_head(p, i);
    return rate_at(p, i, h, self, lane_gather(p, i, h.k, st, T));
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

// The whole warp sets up the trajectory `traj` in column `c` (state, active bits, Fenwick tree);
// returns the total rate on every lane. Groups are processed 32 at a time (chunk): lane l holds
// the sum of group 32 * chunk + l, a scan gives the prefixes, and tree entry
// i = P(i) - P(i - lowbit(i)) (P(x) = sum of groups < x) takes P(i - lowbit(i)) from this chunk
// or, at a multiple of 32, from the chunk boundaries kept one per lane.
__device__ __forceinline__ unsigned long long lane_coop_init(const SimParams& p, const LaneSmem& m, int T, int c,
                                                             unsigned long long traj, unsigned lane) {
    const int n = p.n, G = lane_groups(n);
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
    unsigned long long carry = 0ull, bnd = 0ull;
    for (int ch = 0; ch * 32 < G; ++ch) {
        if ((int)lane == ch) bnd = carry;  // P(32 * ch)
        unsigned long long mine = 0ull;
        const int gend = min(G - ch * 32, 32);
        for (int gg = 0; gg < gend; ++gg) {
            const int g = ch * 32 + gg;
            const int i = g * 32 + (int)lane;
            const unsigned long long v = i < n ? lane_eval(p, i, st, T) : 0ull;
            const unsigned a = __ballot_sync(MBG_FULL, v != 0ull);
            const unsigned long long s = warp_sum_u64(v);
            if (lane == 0u) m.act[(size_t)g * T + c] = a;
            if ((int)lane == gg) mine = s;
        }
        const unsigned long long P = carry + warp_scan_u64(mine, lane);  // P(32 * ch + lane + 1)
        const int idx = ch * 32 + (int)lane + 1;                        // tree index
        const int j = idx - (idx & -idx);
        const unsigned long long v_in = __shfl_sync(MBG_FULL, P, (j - 1 - ch * 32) & 31);
        const unsigned long long v_bnd = __shfl_sync(MBG_FULL, bnd, (j >> 5) & 31);
        const unsigned long long Pj = j > ch * 32 ? v_in : v_bnd;
        if (idx <= G) m.fen[(size_t)(idx - 1) * T + c] = P - Pj;
        carry = __shfl_sync(MBG_FULL, P, 31);
    }
    __syncwarp();
    return carry;
}

// First node whose inclusive rate prefix exceeds r (r < total), or -1.
__device__ __forceinline__ int lane_pick(const SimParams& p, const unsigned* st, const unsigned* act,
                                         const unsigned long long* fen, int T, int G, int top,
                                         unsigned long long r) {
    const int g = fen_find(fen, T, G, top, r);
    if (g >= G) return -1;
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
// `col`: dependency entry e = (dn << 16) | (k_dn << 8) | pos (pos 0xFF: dn itself flipped).
// Patches the active bits and the Fenwick tree (with shared-memory atomics when several lanes may
// patch the same trajectory), returns the rate change and sets `out` when dn is an output node
// whose rate changed.
template <bool ATOMIC>
__device__ __forceinline__ unsigned long long lane_reader(const SimParams& p, unsigned e, const LaneSmem& m, int T,
                                                          int G, int col, bool& out) {
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
    if (a_new != a_old) {
        unsigned* aw = m.act + (size_t)g * T + col;
        if (ATOMIC) atomicXor(aw, 1u << (dn & 31));
        else *aw ^= 1u << (dn & 31);
    }
    const unsigned long long delta = r_new - r_old;
    if (delta != 0ull) {
        if (ATOMIC) fen_add_atomic(m.fen + col, T, G, g, delta);
        else fen_add(m.fen + col, T, G, g, delta);
        out |= __ldg(p.out_pos + dn) >= 0;
    }
    return delta;
}

// After node k flipped in this lane's trajectory: re-evaluates every node whose rate reads k (and
// k itself) in turn. Returns whether an output node's rate changed.
__device__ __forceinline__ bool lane_update(const SimParams& p, int k, const LaneSmem& m, int T, int G, int col,
                                            unsigned long long& total) {
    const int d0 = (int)__ldg(p.dep_off + k), d1 = (int)__ldg(p.dep_off + k + 1);
    bool out = false;
    for (int q = d0; q < d1; ++q) total += lane_reader<false>(p, __ldg(p.deps + q), m, T, G, col, out);
    return out;
}

// Warp-cooperative form of lane_update for every lane at once (k < 0: nothing flipped): the
// reader lists of the 32 flipped nodes are concatenated and dealt out one entry per lane, so a
// step costs ceil(total length / 32) rounds instead of the longest list. Entries of one trajectory
// patch its shared-memory rows with atomics; lanes whose output-node rates changed are marked in
// the warp's wtouch word. The owners read their new totals from their trees afterwards.
__device__ __forceinline__ void lane_coop_update(const SimParams& p, const LaneSmem& m, int T, int G, int wbase,
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
    unsigned touched = 0u;
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
        bool out = false;
        if (q < C) lane_reader<true>(p, __ldg(p.deps + o_d0 + (q - o_ex)), m, T, G, wbase + o, out);
        touched |= __reduce_or_sync(MBG_FULL, out ? 1u << o : 0u);
    }
    if (lane == 0u) m.wtouch[wbase >> 5] = touched;
    __syncwarp();
}

template <bool COOP>
__device__ void sim_lane_body(const SimParams& p, unsigned char* smem) {
    const int T = (int)blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const int wbase = (int)(threadIdx.x & ~31u);
    const int G = lane_groups(p.n);
    const int top = 1 << (31 - __clz(G));
    const LaneSmem m = lane_smem_at(smem, p.n, T);
    const int col = (int)threadIdx.x;
    unsigned* st = m.st + col;
    const unsigned* act = m.act + col;
    const unsigned long long* fen = m.fen + col;

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
                    k = lane_pick(p, st, act, fen, T, G, top, pick_target(d.y, d.z, total));
                    if (k < 0 || k >= p.n) {
                        k = -1;
                        status = TRAJ_ERROR;
                        atomicOr(p.error_flag, (unsigned)DEV_ERR_PICK);
                    } else {
                        st[(k >> 5) * T] ^= 1u << (k & 31);
                        if (!COOP && lane_update(p, k, m, T, G, col, total)) h = lane_entropy(p, st, act, T);
                    }
                }
            }
        }
        if (COOP) {
            lane_coop_update(p, m, T, G, wbase, lane, k);
            if (k >= 0) {
                total = fen_total(fen, T, G);
                if ((m.wtouch[wbase >> 5] >> lane) & 1u) h = lane_entropy(p, st, act, T);
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
