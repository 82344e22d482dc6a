// One trajectory per lane, table-driven, with the state in shared memory and every rate kept
// up to date incrementally (the "lane" layout).
//
// The reference re-evaluates all N rates and scans them on every step
// (src/jit_kernels/simulation.cu:9-21 and 77-164 with the generated compute_transition_rates of
// src/generator.cpp:124-144). Here a lane keeps, for its trajectory:
//   fen[L]  a Fenwick tree over the exact 64-bit fixed-point rate sums of leaves of
//           2^shift 32-node groups (L = ceil(W / 2^shift)): entry i (1-based) holds the
//           sum of leaves (i - lowbit(i), i],
//   st[W]   state words,
//   act[W]  active words (bit i: node i's rate is non-zero),
// in shared memory, in rows of blockDim.x entries (entry [row][thread]), so that the 32 lanes of a
// warp always touch 32 distinct banks whatever rows they read. A step descends the tree to the
// leaf holding the target (log2 L loads, the same count on every lane), then walks the active
// nodes of that leaf's groups in node order: the reference's first-prefix pick, exactly. A
// flip of node k re-evaluates only the nodes whose rate reads k (the dependency CSR) and adds each
// rate change along its leaf's tree path. A new trajectory is set up by the whole warp at once (one node per
// lane), because that pass is O(N).
// Includes nothing: sim_types.h, philox.h, sim_core.cuh and sim_warp.cuh come first.
#pragma once

namespace mbg {

__host__ __device__ __forceinline__ int lane_groups(int n) { return (n + 31) >> 5; }
// Fenwick leaves: 2^shift consecutive 32-node groups each. Wider leaves shrink the tree (and a
// trajectory's shared memory) but lengthen the walk, so they pay only where shared memory rather
// than registers limits the resident trajectories: beyond 16 groups (512 nodes) of the largest
// model a launch holds.
__host__ __device__ __forceinline__ int lane_leaf_shift(int groups) { return groups > 16 ? 1 : 0; }
__host__ __device__ __forceinline__ int lane_leaves(int groups, int shift) {
    return (groups + (1 << shift) - 1) >> shift;
}
// Shared-memory bytes per thread.
__host__ __device__ __forceinline__ unsigned lane_smem_bytes(int n) {
    const int G = lane_groups(n);
    return 8u * (unsigned)G + 8u * (unsigned)lane_leaves(G, lane_leaf_shift(G));
}
struct LaneSmem {
    unsigned long long* fen;  // [L][T]
    unsigned* st;             // [G][T]
    unsigned* act;            // [G][T]
    int shift;                // leaves of 2^shift groups
};

// `G` rows of T entries per array: the largest model's group count in a batched launch, which
// also sets the leaf width of every trajectory of the launch. `act_rows`, when given, holds the
// active-word rows instead of the space after the state rows.
__device__ __forceinline__ LaneSmem lane_smem_at(unsigned char* base, int G, int T, unsigned* act_rows = nullptr) {
    LaneSmem m;
    m.shift = lane_leaf_shift(G);
    m.fen = reinterpret_cast<unsigned long long*>(base);
    m.st = reinterpret_cast<unsigned*>(m.fen + (size_t)lane_leaves(G, m.shift) * T);
    m.act = act_rows ? act_rows : m.st + (size_t)G * T;
    return m;
}

// Bit i of a per-thread bit vector stored as rows of T words (`col` points at the thread's entry
// of row 0).
__device__ __forceinline__ unsigned col_bit(const unsigned* col, int T, int i) {
    return (col[(i >> 5) * T] >> (i & 31)) & 1u;
}

// Fenwick tree of one trajectory over G leaves (`col` points at its entry of row 0; tree index i is
// row i-1).
__device__ __forceinline__ void fen_add(unsigned long long* col, int T, int G, int g, unsigned long long delta) {
    for (int i = g + 1; i <= G; i += i & -i) col[(size_t)(i - 1) * T] += delta;
}
__device__ __forceinline__ void fen_add_atomic(unsigned long long* col, int T, int G, int g,
                                               unsigned long long delta) {
    for (int i = g + 1; i <= G; i += i & -i) atomicAdd(col + (size_t)(i - 1) * T, delta);
}
// Leaf holding target r (r < total): the largest l with sum(leaves < l) <= r; r becomes relative
// to that leaf. `top` is the largest power of two <= G (the tree's size), or half of it when that
// entry is the root.
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

// Table bit of a two-valued node over 5..12 regulators (kLaneWideTable): regulators 0..3 from its
// LaneNode's second half rb, the rest and the table (inline up to 6 regulators) from its LaneWide
// entry.
__device__ __forceinline__ unsigned lane_wide_bit(const SimParams& p, uint4 rb, int k, unsigned self,
                                                  const unsigned* st, int T) {
    const uint4* w = reinterpret_cast<const uint4*>(p.lwide + rb.x);
    const uint4 w0 = __ldg(w), w1 = __ldg(w + 1);
    unsigned idx = lane_idx4(st, T, 4, rb.y, rb.z) | (lane_idx4(st, T, min(k - 4, 4), w0.x, w0.y) << 4);
    if (k > 8) idx |= lane_idx4(st, T, k - 8, w0.z, w0.w) << 8;
    const unsigned a = (self << k) | idx;
    unsigned word;
    if (k <= 6) {
        const unsigned q = a >> 5;
        word = q == 0u ? w1.x : q == 1u ? w1.y : q == 2u ? w1.z : w1.w;
    } else {
        word = __ldg(p.tabs + w1.x + (a >> 5));
    }
    return (word >> (a & 31u)) & 1u;
}

// Rate of node i in the state column st, evaluated from its tables. FULL: the model may have
// multi-valued (palette) rates or nodes over more than 12 regulators; without them those paths
// are left out of the kernel (a smaller loop body).
template <bool FULL>
__device__ __forceinline__ unsigned long long lane_eval(const SimParams& p, int i, const unsigned* st, int T) {
    const uint4* rec = reinterpret_cast<const uint4*>(p.lnodes + i);
    const uint4 ra = __ldg(rec), rb = __ldg(rec + 1);
    const unsigned self = col_bit(st, T, i);
    const unsigned flags = rb.w >> 16;
    if (flags == 0u || flags == kLaneWideTable) {
        const int k = (int)(rb.w & 0xffffu);
        const unsigned on = flags == 0u ? (rb.x >> ((self << k) | lane_idx4(st, T, k, rb.y, rb.z))) & 1u
                                        : lane_wide_bit(p, rb, k, self, st, T);
        if (!on) return 0ull;
        return self ? (((unsigned long long)ra.w << 32) | ra.z) : (((unsigned long long)ra.y << 32) | ra.x);
    }
    if (!FULL) return 0ull;
    const NodeHead h = load_head(p, i);
    return rate_at(p, i, h, self, lane_gather(p, i, h.k, st, T));
}

// Current rate of node i from its active bit (BINARY) or its table (PALETTE).
template <bool FULL>
__device__ __forceinline__ unsigned long long lane_rate(const SimParams& p, int i, const unsigned* st,
                                                        const unsigned* act, int T) {
    const unsigned self = col_bit(st, T, i);
    if (FULL && p.has_palette && (__ldg(&p.lnodes[i].flags) & kLanePalette)) {
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
template <bool FULL>
__device__ __forceinline__ float lane_entropy(const SimParams& p, const unsigned* st, const unsigned* act, int T) {
    unsigned long long R = 0ull;
    float c = 0.f;
    for (int q = 0; q < p.n_out; ++q) {
        const unsigned long long r = lane_rate<FULL>(p, __ldg(p.out_nodes + q), st, act, T);
        if (r) {
            R += r;
            const float rr = u64_to_f32(r) * p.to_real;
            c += rr * __log2f(rr);
        }
    }
    return entropy_from_sums(R, c, p.to_real);
}

// The whole warp sets up the trajectory `traj` in column `c` (state, active bits, Fenwick tree);
// returns the total rate on every lane. Leaves are processed 32 at a time (chunk): lane l holds
// the sum of leaf 32 * chunk + l, a scan gives the prefixes, and tree entry
// i = P(i) - P(i - lowbit(i)) (P(x) = sum of leaves < x) takes P(i - lowbit(i)) from this chunk
// or, at a multiple of 32, from the chunk boundaries kept one per lane.
template <bool FULL>
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
    const int L = lane_leaves(G, m.shift);
    unsigned long long carry = 0ull, bnd = 0ull;
    for (int ch = 0; ch * 32 < L; ++ch) {
        if ((int)lane == ch) bnd = carry;  // P(32 * ch)
        unsigned long long mine = 0ull;
        const int lend = min(L - ch * 32, 32);
        for (int ll = 0; ll < lend; ++ll) {
            // leaf ch * 32 + ll: its groups in turn, one node per lane
            unsigned long long v = 0ull;
            for (int h = 0; h < (1 << m.shift); ++h) {
                const int g = ((ch * 32 + ll) << m.shift) + h;
                if (g >= G) break;
                const int i = g * 32 + (int)lane;
                const unsigned long long vi = i < n ? lane_eval<FULL>(p, i, st, T) : 0ull;
                const unsigned a = __ballot_sync(MBG_FULL, vi != 0ull);
                if (lane == 0u) m.act[(size_t)g * T + c] = a;
                v += vi;
            }
            const unsigned long long s = warp_sum_u64(v);
            if ((int)lane == ll) mine = s;
        }
        const unsigned long long P = carry + warp_scan_u64(mine, lane);  // P(32 * ch + lane + 1)
        const int idx = ch * 32 + (int)lane + 1;                        // tree index
        const int j = idx - (idx & -idx);
        const unsigned long long v_in = __shfl_sync(MBG_FULL, P, (j - 1 - ch * 32) & 31);
        const unsigned long long v_bnd = __shfl_sync(MBG_FULL, bnd, (j >> 5) & 31);
        const unsigned long long Pj = j > ch * 32 ? v_in : v_bnd;
        if (idx <= L) m.fen[(size_t)(idx - 1) * T + c] = P - Pj;
        carry = __shfl_sync(MBG_FULL, P, 31);
    }
    __syncwarp();
    return carry;
}

// Walks the active nodes of group g in node order: the first whose inclusive rate prefix exceeds
// r, or -1 with r reduced by the group's total.
template <bool FULL>
__device__ __forceinline__ int lane_walk(const SimParams& p, const unsigned* st, const unsigned* act, int T, int g,
                                         unsigned long long& r) {
    unsigned aw = act[g * T];
    const unsigned sw = st[g * T];
    if (!FULL || !p.has_palette) {
        // the next eight active nodes' rates are loaded together, then compared in node order
        const unsigned long long* rates = &p.lnodes[g * 32].up;  // 4 words per LaneNode
        while (aw) {
            int b[8];
            unsigned long long v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                b[u] = aw ? __ffs(aw) - 1 : -1;
                aw &= aw - 1u;
                v[u] = b[u] >= 0 ? __ldg(rates + 4 * b[u] + ((sw >> (b[u] & 31)) & 1u)) : 0ull;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (b[u] < 0) return -1;
                if (r < v[u]) return g * 32 + b[u];
                r -= v[u];
            }
        }
        return -1;
    }
    while (aw) {
        const int b = __ffs(aw) - 1;
        aw &= aw - 1u;
        const int i = g * 32 + b;
        const unsigned long long v =
            p.has_palette ? lane_rate<FULL>(p, i, st, act, T) : __ldg(&p.lnodes[i].up + ((sw >> b) & 1u));
        if (r < v) return i;
        r -= v;
    }
    return -1;
}

// First node whose inclusive rate prefix exceeds r (r < total), or -1: the leaf from the tree,
// then its groups in turn. SPLIT writes the two walks of a two-group leaf out separately instead
// of as a loop: the same result, different code; which one runs faster depends on the kernel it
// is compiled into (measured per kernel).
template <bool SPLIT, bool FULL>
__device__ __forceinline__ int lane_pick(const SimParams& p, const unsigned* st, const unsigned* act,
                                         const unsigned long long* fen, int T, int G, int shift, int top,
                                         unsigned long long r) {
    const int l = fen_find(fen, T, lane_leaves(G, shift), top, r);
    if (SPLIT) {
        const int g = l << shift;
        if (g >= G) return -1;
        const int k = lane_walk<FULL>(p, st, act, T, g, r);
        if (k >= 0 || shift == 0 || g + 1 >= G) return k;
        return lane_walk<FULL>(p, st, act, T, g + 1, r);
    }
    for (int h = 0; h < (1 << shift); ++h) {
        const int g = (l << shift) + h;
        if (g >= G) return -1;
        const int k = lane_walk<FULL>(p, st, act, T, g, r);
        if (k >= 0) return k;
    }
    return -1;
}

// Re-evaluates reader dn of a node that just flipped, in the trajectory whose entries start at
// `col`: dependency entry e = (dn << 16) | (out << 15) | (k_dn << 8) | pos (pos 0xFF: dn itself
// flipped).
// Patches the active bits and the Fenwick tree (with shared-memory atomics when several lanes may
// patch the same trajectory), returns the rate change and sets `out` when dn is an output node
// whose rate changed.
template <bool ATOMIC, bool FULL>
__device__ __forceinline__ unsigned long long lane_reader_rec(const SimParams& p, unsigned e, uint4 ra, uint4 rb,
                                                              const LaneSmem& m, int T, int col, bool& out) {
    const int dn = (int)(e >> 16);
    const int kd = (int)((e >> 8) & 0x7fu);
    const unsigned pos = e & 0xffu;
    const unsigned* st = m.st + col;
    const unsigned self = col_bit(st, T, dn);
    const unsigned self_old = pos == 0xffu ? self ^ 1u : self;
    const unsigned flags = rb.w >> 16;
    unsigned long long r_new, r_old;
    unsigned a_new, a_old;
    if (!FULL || !(flags & kLanePalette)) {
        if (flags == 0u) {
            // up to 4 regulators and their table in the record itself
            a_new = (rb.x >> ((self << kd) | lane_idx4(st, T, kd, rb.y, rb.z))) & 1u;
        } else if (!FULL || flags == kLaneWideTable) {
            a_new = lane_wide_bit(p, rb, kd, self, st, T);
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
        const int L = lane_leaves(lane_groups(p.n), m.shift);
        if (ATOMIC) fen_add_atomic(m.fen + col, T, L, g >> m.shift, delta);
        else fen_add(m.fen + col, T, L, g >> m.shift, delta);
        out |= ((e >> 15) & 1u) != 0u;
    }
    return delta;
}

template <bool ATOMIC, bool FULL>
__device__ __forceinline__ unsigned long long lane_reader(const SimParams& p, unsigned e, const LaneSmem& m, int T,
                                                          int col, bool& out) {
    const uint4* rec = reinterpret_cast<const uint4*>(p.lnodes + (e >> 16));
    return lane_reader_rec<ATOMIC, FULL>(p, e, __ldg(rec), __ldg(rec + 1), m, T, col, out);
}

// After node k flipped in this lane's trajectory: re-evaluates every node whose rate reads k (and
// k itself) in turn. Returns whether an output node's rate changed.
template <bool FULL>
__device__ __forceinline__ bool lane_update(const SimParams& p, int k, const LaneSmem& m, int T, int col,
                                            unsigned long long& total) {
    const int d0 = (int)__ldg(p.dep_off + k), d1 = (int)__ldg(p.dep_off + k + 1);
    bool out = false;
    // the next reader's dependency entry and record are fetched while this one is applied
    unsigned e = __ldg(p.deps + d0);
    uint4 ra = __ldg(reinterpret_cast<const uint4*>(p.lnodes + (e >> 16)));
    uint4 rb = __ldg(reinterpret_cast<const uint4*>(p.lnodes + (e >> 16)) + 1);
    for (int q = d0; q < d1; ++q) {
        unsigned e2 = 0u;
        uint4 ra2 = ra, rb2 = rb;
        if (q + 1 < d1) {
            e2 = __ldg(p.deps + q + 1);
            ra2 = __ldg(reinterpret_cast<const uint4*>(p.lnodes + (e2 >> 16)));
            rb2 = __ldg(reinterpret_cast<const uint4*>(p.lnodes + (e2 >> 16)) + 1);
        }
        total += lane_reader_rec<false, FULL>(p, e, ra, rb, m, T, col, out);
        e = e2;
        ra = ra2;
        rb = rb2;
    }
    return out;
}

// Warp-cooperative form of lane_update for every lane at once (k < 0: nothing flipped): the
// reader lists of the 32 flipped nodes are concatenated and dealt out one entry per lane, so a
// step costs ceil(total length / 32) rounds instead of the longest list. Entries of one trajectory
// patch its shared-memory rows with atomics. Returns (on every lane) the mask of lanes whose
// output-node rates changed. `owner(o)` gives the model of lane o's trajectory (called by all
// lanes).
template <bool FULL, class Owner>
__device__ __forceinline__ unsigned lane_coop_update(const SimParams& mine, Owner owner, const LaneSmem& m, int T,
                                                 int wbase, unsigned lane, int k) {
    int d0 = 0, c = 0;
    if (k >= 0) {
        d0 = (int)__ldg(mine.dep_off + k);
        c = (int)__ldg(mine.dep_off + k + 1) - d0;
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
        const SimParams& po = owner(o);
        bool out = false;
        if (q < C) lane_reader<true, FULL>(po, __ldg(po.deps + o_d0 + (q - o_ex)), m, T, wbase + o, out);
        touched |= __reduce_or_sync(MBG_FULL, out ? 1u << o : 0u);
    }
    __syncwarp();  // every patch is visible to its trajectory's lane
    return touched;
}

// Registers of the trajectory a lane is running.
struct LaneTraj {
    unsigned long long j = 0, step = 0, t = 0, t1 = 0, total = 0;
    unsigned trans = 0, so = 0;
    float h = 0.f;
    unsigned char status = TRAJ_CONTINUE;
    bool have = false, done = false;
    WindowAcc acc;
};

// End-state counts of one lane (or warp) until they are added to a counter block.
struct LaneCounts {
    unsigned long long trans = 0, steps = 0;
    unsigned fin = 0, fix = 0, lim = 0, err = 0;
    __device__ __forceinline__ void flush(unsigned long long* counters) {
        if (trans) atomicAdd(counters + CNT_TRANSITIONS, trans);
        if (steps) atomicAdd(counters + CNT_STEPS, steps);
        if (fin) atomicAdd(counters + CNT_FINISHED, (unsigned long long)fin);
        if (fix) atomicAdd(counters + CNT_FIXED, (unsigned long long)fix);
        if (lim) atomicAdd(counters + CNT_STEP_LIMIT, (unsigned long long)lim);
        if (err) atomicAdd(counters + CNT_ERROR, (unsigned long long)err);
        *this = LaneCounts();
    }
    // all lanes of the warp: one atomic per counter
    __device__ __forceinline__ void flush_warp(unsigned long long* counters, unsigned lane) {
        for (int o = 16; o > 0; o >>= 1) {
            trans += __shfl_xor_sync(MBG_FULL, trans, o);
            steps += __shfl_xor_sync(MBG_FULL, steps, o);
        }
        fin = __reduce_add_sync(MBG_FULL, fin);
        fix = __reduce_add_sync(MBG_FULL, fix);
        lim = __reduce_add_sync(MBG_FULL, lim);
        err = __reduce_add_sync(MBG_FULL, err);
        if (lane == 0u) flush(counters);
    }
};

// A new trajectory's registers once its state is set up.
template <bool FULL>
__device__ __forceinline__ void lane_begin(const SimParams& p, const LaneSmem& m, int T, int col, LaneTraj& tr) {
    tr.have = true;
    tr.t = 0;
    tr.step = 0;
    tr.trans = 0;
    tr.so = lane_out_index(p, m.st + col, T);
    tr.h = lane_entropy<FULL>(p, m.st + col, m.act + col, T);
    win_begin(tr.acc, p, tr.so);
}

// One Gillespie step up to the flip (src/jit_kernels/simulation.cu:104-147): fixed point, step
// cap, dt and window accumulation, end of time, pick and flip. Returns the flipped node or -1;
// tr.status says whether the trajectory ended. Without `coop` the readers are updated here.
template <bool SPLIT, bool FULL>
__device__ __forceinline__ int lane_step_front(const SimParams& p, const LaneSmem& m, int T, int col, LaneTraj& tr,
                                               bool coop) {
    tr.status = TRAJ_CONTINUE;
    if (tr.total == 0ull) {
        if (p.discrete) win_discrete(p, tr.step, tr.so, 0.f, true);
        else win_slice(tr.acc, p, tr.t, p.max_time_fx, tr.so, 0.f, true);
        tr.t = p.max_time_fx;
        tr.status = TRAJ_FIXED_POINT;
        return -1;
    }
    if (tr.step >= p.max_steps) {
        tr.status = TRAJ_STEP_LIMIT;
        return -1;
    }
    const u32x4 d = philox_step(p.seed, p.traj_base + tr.j, tr.step);
    tr.t1 = next_time(p, tr.t, tr.step, p.discrete ? 0.f : neg_log_u(d.x), tr.total);
    if (p.discrete) win_discrete(p, tr.step, tr.so, tr.h, true);
    else win_slice(tr.acc, p, tr.t, tr.t1, tr.so, tr.h, true);
    ++tr.step;
    if (tr.t1 >= p.max_time_fx) {
        tr.t = p.max_time_fx;
        tr.status = TRAJ_FINISHED;
        return -1;
    }
    const int G = lane_groups(p.n), L = lane_leaves(G, m.shift);
    unsigned* st = m.st + col;
    // the tree's root (L a power of two) holds the total, which r never reaches: start below it
    const int top = 1 << (31 - __clz(L));
    const int k = lane_pick<SPLIT, FULL>(p, st, m.act + col, m.fen + col, T, G, m.shift, top == L ? top >> 1 : top,
                            pick_target(d.y, d.z, tr.total));
    if (k < 0 || k >= p.n) {
        tr.status = TRAJ_ERROR;
        atomicOr(p.error_flag, (unsigned)DEV_ERR_PICK);
        return -1;
    }
    st[(k >> 5) * T] ^= 1u << (k & 31);
    if (!coop && lane_update<FULL>(p, k, m, T, col, tr.total)) tr.h = lane_entropy<FULL>(p, st, m.act + col, T);
    return k;
}

// After the readers of k were updated cooperatively: the new total from the tree, the entropy
// when an output node's rate changed.
template <bool FULL>
__device__ __forceinline__ void lane_after_coop(const SimParams& p, const LaneSmem& m, int T, int col,
                                                unsigned touched, unsigned lane, LaneTraj& tr) {
    tr.total = fen_total(m.fen + col, T, lane_leaves(lane_groups(p.n), m.shift));
    if ((touched >> lane) & 1u) tr.h = lane_entropy<FULL>(p, m.st + col, m.act + col, T);
}

// Completes the step: output state, clock, transition count; at the end of the trajectory its
// window run, final state, optional records, fixed point and counts.
__device__ __forceinline__ void lane_step_back(const SimParams& p, const LaneSmem& m, int T, int col, LaneTraj& tr,
                                               int k, LaneCounts& c) {
    if (k >= 0) {
        const short op = __ldg(p.out_pos + k);
        if (op >= 0) tr.so ^= 1u << op;
        tr.t = tr.t1;
        ++tr.trans;
    }
    const unsigned char status = tr.status;
    if (status == TRAJ_CONTINUE) return;
    const unsigned* st = m.st + col;
    if (!p.discrete && status != TRAJ_ERROR) win_end(tr.acc, p, tr.t, true);
    c.trans += tr.trans;
    c.steps += tr.step + (status == TRAJ_FIXED_POINT ? 1 : 0);
    c.fin += status == TRAJ_FINISHED;
    c.fix += status == TRAJ_FIXED_POINT;
    c.lim += status == TRAJ_STEP_LIMIT;
    c.err += status == TRAJ_ERROR;
    record_end_scalar(p, tr.j, status, tr.t, tr.trans, tr.so);
    if (p.traj_state)
        for (int w = 0; w < p.words; ++w) p.traj_state[tr.j * p.words + w] = st[w * T];
    if (status == TRAJ_FIXED_POINT) {
        const unsigned slot = atomicAdd(p.fp_count, 1u);
        if (slot < p.fp_capacity) {
            for (int w = 0; w < p.words; ++w) p.fp_states[(unsigned long long)slot * p.words + w] = st[w * T];
        } else {
            atomicOr(p.error_flag, (unsigned)DEV_ERR_FP_OVERFLOW);
        }
    }
    tr.have = false;
}

// One simulation: lanes take trajectory ids from the run's work counter.
template <bool COOP, bool FULL>
__device__ void sim_lane_body(const SimParams& p, unsigned char* smem, unsigned* act_rows = nullptr) {
    const int T = (int)blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const int wbase = (int)(threadIdx.x & ~31u);
    const LaneSmem m = lane_smem_at(smem, lane_groups(p.n), T, act_rows);
    const int col = (int)threadIdx.x;
    LaneTraj tr;
    LaneCounts c;
    for (;;) {
        const unsigned need = __ballot_sync(MBG_FULL, !tr.have && !tr.done);
        if (need) {
            unsigned long long base = 0;
            const int leader = __ffs(need) - 1;
            if ((int)lane == leader) base = atomicAdd(p.counters + CNT_WORK, (unsigned long long)__popc(need));
            base = __shfl_sync(MBG_FULL, base, leader);
            bool start = false;
            if (!tr.have && !tr.done) {
                tr.j = base + __popc(need & ((1u << lane) - 1u));
                if (tr.j < p.n_traj) start = true;
                else tr.done = true;
            }
            unsigned init = __ballot_sync(MBG_FULL, start);
            while (init) {
                const int L = __ffs(init) - 1;
                init &= init - 1u;
                const unsigned long long jl = __shfl_sync(MBG_FULL, tr.j, L);
                const unsigned long long tot = lane_coop_init<FULL>(p, m, T, wbase + L, p.traj_base + jl, lane);
                if ((int)lane == L) tr.total = tot;
            }
            if (start) lane_begin<FULL>(p, m, T, col, tr);
        }
        if (__all_sync(MBG_FULL, tr.done)) break;
        if (!COOP && !tr.have) continue;
        const int k = tr.have ? lane_step_front<false, FULL>(p, m, T, col, tr, COOP) : -1;
        if (COOP) {
            const unsigned touched =
                lane_coop_update<FULL>(p, [&](int) -> const SimParams& { return p; }, m, T, wbase, lane, k);
            if (k >= 0) lane_after_coop<FULL>(p, m, T, col, touched, lane, tr);
        }
        if (tr.have) lane_step_back(p, m, T, col, tr, k, c);
    }
    c.flush_warp(p.counters, lane);
}

// Many instances in one launch (batched sweeps): lanes take work items from one counter over the
// instances' trajectory counts; each lane runs its item with its instance's model and adds its
// counts to that instance's counters when it moves to another instance. Shared memory has rows
// for the largest instance of the launch (b.rows groups).
template <bool COOP, bool FULL>
__device__ void sim_lane_batch_body(const BatchDesc& b, unsigned char* smem, unsigned* act_rows = nullptr) {
    const int T = (int)blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const int wbase = (int)(threadIdx.x & ~31u);
    const LaneSmem m = lane_smem_at(smem, b.rows, T, act_rows);
    const int col = (int)threadIdx.x;
    const unsigned long long items = __ldg(b.prefix + b.n_inst);
    const SimParams* pp = b.params;
    int cur = -1;
    LaneTraj tr;
    LaneCounts c;
    for (;;) {
        const unsigned need = __ballot_sync(MBG_FULL, !tr.have && !tr.done);
        if (need) {
            unsigned long long base = 0;
            const int leader = __ffs(need) - 1;
            if ((int)lane == leader) base = atomicAdd(b.work, (unsigned long long)__popc(need));
            base = __shfl_sync(MBG_FULL, base, leader);
            bool start = false;
            if (!tr.have && !tr.done) {
                const unsigned long long w = base + __popc(need & ((1u << lane) - 1u));
                if (w < items) {
                    int lo = 0, hi = b.n_inst;  // prefix[lo] <= w < prefix[hi]
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (__ldg(b.prefix + mid) <= w) lo = mid;
                        else hi = mid;
                    }
                    if (lo != cur) {
                        if (cur >= 0) c.flush(b.params[cur].counters);
                        cur = lo;
                    }
                    pp = b.params + lo;
                    tr.j = w - __ldg(b.prefix + lo);
                    start = true;
                } else {
                    tr.done = true;
                }
            }
            unsigned init = __ballot_sync(MBG_FULL, start);
            while (init) {
                const int L = __ffs(init) - 1;
                init &= init - 1u;
                const SimParams* pl = reinterpret_cast<const SimParams*>(
                    __shfl_sync(MBG_FULL, reinterpret_cast<unsigned long long>(pp), L));
                const unsigned long long jl = __shfl_sync(MBG_FULL, tr.j, L);
                const unsigned long long tot = lane_coop_init<FULL>(*pl, m, T, wbase + L, pl->traj_base + jl, lane);
                if ((int)lane == L) tr.total = tot;
            }
            if (start) lane_begin<FULL>(*pp, m, T, col, tr);
        }
        if (__all_sync(MBG_FULL, tr.done)) break;
        if (!COOP && !tr.have) continue;
        const SimParams& p = *pp;
        const int k = tr.have ? lane_step_front<true, FULL>(p, m, T, col, tr, COOP) : -1;
        if (COOP) {
            const unsigned touched = lane_coop_update<FULL>(
                p,
                [&](int o) -> const SimParams& {
                    return *reinterpret_cast<const SimParams*>(
                        __shfl_sync(MBG_FULL, reinterpret_cast<unsigned long long>(pp), o));
                },
                m, T, wbase, lane, k);
            if (k >= 0) lane_after_coop<FULL>(p, m, T, col, touched, lane, tr);
        }
        if (tr.have) lane_step_back(p, m, T, col, tr, k, c);
    }
    if (cur >= 0) c.flush(b.params[cur].counters);
}

}  // namespace mbg
