// Warp-per-trajectory kernel for networks of hundreds to tens of thousands of nodes.
//
// One warp owns one trajectory. Rates are exact 64-bit fixed point, grouped by 32 nodes (L1,
// N/32 groups) and by 1024 nodes (L2, N/1024 blocks; N <= 32768). The top level of that tree
// (the L1 groups when N <= 1024, else the L2 blocks) lives in registers as an inclusive prefix
// sum, lane i holding the sum over top entries 0..i; the L1 groups of larger models live in
// shared memory. Shared memory also holds the state words, one "active" bit per node (rate != 0)
// and, in the cached-index variant, each node's current regulator index. Per transition:
//   pick    __ballot over the register prefix (no scan); for N > 1024 a warp scan (__shfl_up) of
//           the 32 L1 sums of the chosen block; then a warp scan of the 32 leaf rates of the
//           chosen group, each leaf rate read from two bits and the node's two rate values;
//   flip    one shared-memory word;
//   update  the nodes that read the flipped node (CSR `deps`, which carries the bit position of
//           the flipped node in each reader's index) are re-evaluated one per lane: the cached
//           index is patched with one XOR and looked up in the node's truth table; the exact
//           difference of old and new rate is broadcast lane to lane into the register prefix
//           (and added to L1 with a shared atomic), so the sums never drift.
// The Philox draws of 32 consecutive steps are computed at once, one step per lane, and handed
// out with __shfl, so the generator's latency is paid once per 32 steps.
// The reference instead recomputes all N rates into a thread-local array every step and scans
// it linearly (src/generator.cpp:124-144, src/jit_kernels/simulation.cu:9-21).
#pragma once

namespace mbg {

struct WarpSmem {
    unsigned long long* l1;  // N > 1024 only
    unsigned* st;            // state words
    unsigned* act;           // active bits
    unsigned* idx;           // cached regulator index per node (cached-index variant)
};

__host__ __device__ __forceinline__ int warp_groups(int n) { return (n + 31) >> 5; }
__host__ __device__ __forceinline__ int warp_groups2(int n) { return (warp_groups(n) + 31) >> 5; }
__host__ __device__ __forceinline__ int warp_words_padded(int n) { return ((((n + 31) >> 5) + 3) >> 2) << 2; }
__host__ __device__ __forceinline__ int warp_l1_smem(int n) { return warp_groups(n) > 32 ? warp_groups(n) : 0; }
// shared-memory bytes per warp: L1 (8 B each, N > 1024) + state and active words + cached index
__host__ __device__ __forceinline__ unsigned warp_smem_bytes(int n, bool cached_index) {
    return (unsigned)(8 * warp_l1_smem(n) + 8 * warp_words_padded(n) + (cached_index ? 4 * (((n + 3) >> 2) << 2) : 0));
}

struct NodeHead {  // the first 32 bytes of a DevNode
    unsigned long long up, down;
    unsigned tab_off, pal_off;
    int k, kind;
    unsigned reg_off;
};

__device__ __forceinline__ void load_rates(const SimParams& p, int i, unsigned long long& up,
                                           unsigned long long& down) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(p.nodes + i));
    up = ((unsigned long long)a.y << 32) | a.x;
    down = ((unsigned long long)a.w << 32) | a.z;
}

__device__ __forceinline__ NodeHead load_head(const SimParams& p, int i) {
    const uint4* q = reinterpret_cast<const uint4*>(p.nodes + i);
    const uint4 a = __ldg(q), b = __ldg(q + 1);
    NodeHead h;
    h.up = ((unsigned long long)a.y << 32) | a.x;
    h.down = ((unsigned long long)a.w << 32) | a.z;
    h.tab_off = b.x;
    h.pal_off = b.y;
    h.k = (int)(b.z & 0xffffu);
    h.kind = (int)(b.z >> 16);
    h.reg_off = b.w;
    return h;
}

__device__ __forceinline__ unsigned st_bit(const unsigned* st, int i) { return (st[i >> 5] >> (i & 31)) & 1u; }

// Regulator index of a node with k <= 4 regulators packed as r01 = r0 | r1 << 16, r23 likewise.
__device__ __forceinline__ unsigned warp_idx4(const unsigned* st, int k, unsigned r01, unsigned r23) {
    unsigned idx = 0u;
    if (k > 0) idx |= st_bit(st, (int)(r01 & 0xffffu));
    if (k > 1) idx |= st_bit(st, (int)(r01 >> 16)) << 1;
    if (k > 2) idx |= st_bit(st, (int)(r23 & 0xffffu)) << 2;
    if (k > 3) idx |= st_bit(st, (int)(r23 >> 16)) << 3;
    return idx;
}

// Regulator index of node i in state st (bit j = state of its j-th regulator).
__device__ __forceinline__ unsigned gather_regs(const SimParams& p, int i, const NodeHead& h, const unsigned* st) {
    unsigned idx = 0u;
    const unsigned short* inl = p.nodes[i].r;
    const unsigned short* far = p.regs + h.reg_off;
    for (int j = 0; j < h.k; ++j) {
        const int r = j < kInlineRegs ? __ldg(inl + j) : __ldg(far + j);
        idx |= st_bit(st, r) << j;
    }
    return idx;
}

// Whether the rate of BINARY node i (k regulators) is non-zero at entry (self << k) | idx.
__device__ __forceinline__ unsigned table_bit(const SimParams& p, int i, int k, unsigned self, unsigned idx) {
    const unsigned a = (self << k) | idx;
    if (k <= 5) return (unsigned)(__ldg(&p.nodes[i].table) >> a) & 1u;
    const unsigned tab_off = __ldg(&p.nodes[i].tab_off);
    return (__ldg(p.tabs + tab_off + (a >> 5)) >> (a & 31)) & 1u;
}

__device__ __forceinline__ unsigned long long palette_rate(const SimParams& p, const NodeHead& h, unsigned self,
                                                           unsigned idx) {
    const unsigned a = (self << h.k) | idx;
    return __ldg(p.palette + h.pal_off + __ldg(p.pidx + h.tab_off + a));
}

// Rate of node i at regulator index idx and own state self.
__device__ __forceinline__ unsigned long long rate_at(const SimParams& p, int i, const NodeHead& h, unsigned self,
                                                      unsigned idx) {
    if (h.kind == 0) return table_bit(p, i, h.k, self, idx) ? (self ? h.down : h.up) : 0ull;
    return palette_rate(p, h, self, idx);
}

// Current rate of node i from its active bit (BINARY) or its table (PALETTE).
template <bool IDX>
__device__ __forceinline__ unsigned long long current_rate(const SimParams& p, int i, const WarpSmem& m) {
    if (p.has_palette) {
        const NodeHead h = load_head(p, i);
        if (h.kind != 0) return palette_rate(p, h, st_bit(m.st, i), IDX ? m.idx[i] : gather_regs(p, i, h, m.st));
    }
    if (!st_bit(m.act, i)) return 0ull;
    unsigned long long up, down;
    load_rates(p, i, up, down);
    return st_bit(m.st, i) ? down : up;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(MBG_FULL, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum_f32(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(MBG_FULL, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_scan_u64(unsigned long long v, unsigned lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long o = __shfl_up_sync(MBG_FULL, v, d);
        if (lane >= (unsigned)d) v += o;
    }
    return v;
}

// Lane whose inclusive prefix `inc` first exceeds r; r becomes relative to that lane. -1 if none.
__device__ __forceinline__ int prefix_pick(unsigned long long inc, unsigned long long& r) {
    const unsigned b = __ballot_sync(MBG_FULL, inc > r);
    const int j = __ffs(b) - 1;
    const unsigned long long before = __shfl_sync(MBG_FULL, inc, j > 0 ? j - 1 : 0);
    if (j > 0) r -= before;
    return j;
}

// Scan of per-lane values v, then prefix_pick.
__device__ __forceinline__ int warp_pick(unsigned long long v, unsigned long long& r, unsigned lane) {
    return prefix_pick(warp_scan_u64(v, lane), r);
}

// Transition entropy of the current state, -sum p log2 p over the output nodes, one output node
// per lane (generator.cpp:146-175). The warp path requires n_out <= 32.
template <bool IDX>
__device__ __forceinline__ float warp_entropy(const SimParams& p, const WarpSmem& m, unsigned lane) {
    unsigned long long r = 0ull;
    if ((int)lane < p.n_out) r = current_rate<IDX>(p, __ldg(p.out_nodes + lane), m);
    const unsigned long long R = warp_sum_u64(r);
    if (R == 0ull) return 0.f;
    const float pr = __fdividef(u64_to_f32(r), u64_to_f32(R));
    const float term = pr > 0.f ? pr * __log2f(pr) : 0.f;
    const float h = -warp_sum_f32(term);
    return h > 0.f ? h : 0.f;
}

__device__ __forceinline__ unsigned warp_out_index(const SimParams& p, const unsigned* st, unsigned lane) {
    unsigned b = 0u;
    if ((int)lane < p.n_out) b = st_bit(st, __ldg(p.out_nodes + lane));
    return __ballot_sync(MBG_FULL, b != 0u);
}

__device__ __forceinline__ void warp_init_state(const SimParams& p, unsigned long long traj, unsigned* st,
                                                unsigned lane) {
    const int W = p.words;
    for (int w = (int)lane; w < W; w += 32) {
        unsigned word = 0u;
        for (int b = 0; b < 8; ++b) {
            const int blk = w * 8 + b;
            if (4 * blk >= p.n) break;
            const u32x4 d = philox_init(p.seed, traj, (unsigned)blk);
            const unsigned v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int i = 4 * blk + c;
                if (i < p.n && (v[c] >> 8) < __ldg(p.istate_thr + i)) word |= 1u << (i & 31);
            }
        }
        st[w] = word;
    }
    __syncwarp();
}

// Evaluates every node from its table: active bits, cached indices, L1 (N > 1024) and the
// register prefix over the top level; returns this lane's prefix, `total` gets the sum.
template <bool IDX>
__device__ __forceinline__ unsigned long long warp_build_sums(const SimParams& p, const WarpSmem& m, unsigned lane,
                                                              unsigned long long& total) {
    const int G = warp_groups(p.n);
    unsigned long long top = 0ull;
    for (int g = 0; g < G; ++g) {
        const int i = g * 32 + (int)lane;
        unsigned long long v = 0ull;
        if (i < p.n) {
            const NodeHead h = load_head(p, i);
            const unsigned idx = gather_regs(p, i, h, m.st);
            if (IDX) m.idx[i] = idx;
            v = rate_at(p, i, h, st_bit(m.st, i), idx);
        }
        const unsigned a = __ballot_sync(MBG_FULL, v != 0ull);
        const unsigned long long s = warp_sum_u64(v);
        if (lane == 0) {
            m.act[g] = a;
            if (G > 32) m.l1[g] = s;
        }
        if ((int)lane == (G > 32 ? (g >> 5) : g)) top += s;
    }
    __syncwarp();
    const unsigned long long pre = warp_scan_u64(top, lane);
    total = __shfl_sync(MBG_FULL, pre, 31);
    return pre;
}

// Draws of steps base .. base+31, one step per lane.
struct StepDraws {
    unsigned long long base;
    float nlog;  // -ln U of the dt draw
    unsigned y, z;
};

__device__ __forceinline__ void draws_fill(const SimParams& p, unsigned long long traj, unsigned long long base,
                                           unsigned lane, StepDraws& d) {
    const u32x4 r = philox_step(p.seed, traj, base + lane);
    d.base = base;
    d.nlog = p.discrete ? 0.f : neg_log_u(r.x);
    d.y = r.y;
    d.z = r.z;
}

// One trajectory, run by the whole warp. Returns the end status; counts go to the references.
template <bool IDX>
__device__ unsigned char warp_trajectory(const SimParams& p, const WarpSmem& m, unsigned long long j, unsigned lane,
                                         unsigned long long& c_trans, unsigned long long& c_steps) {
    const bool leader = lane == 0u;
    const int G = warp_groups(p.n);
    const bool two_level = G > 32;
    const int top_count = two_level ? warp_groups2(p.n) : G;
    const unsigned long long traj = p.traj_base + j;
    warp_init_state(p, traj, m.st, lane);
    unsigned long long total;
    unsigned long long pre = warp_build_sums<IDX>(p, m, lane, total);
    unsigned so = warp_out_index(p, m.st, lane);
    float h = warp_entropy<IDX>(p, m, lane);
    WindowAcc acc;
    win_begin(acc, p, so);
    StepDraws dr;
    draws_fill(p, traj, 0, lane, dr);
    unsigned long long t = 0, step = 0;
    unsigned trans = 0;
    unsigned char status = TRAJ_CONTINUE;
    for (;;) {
        if (total == 0ull) {
            if (p.discrete) win_discrete(p, step, so, 0.f, leader);
            else win_slice(acc, p, t, p.max_time_fx, so, 0.f, leader);
            t = p.max_time_fx;
            status = TRAJ_FIXED_POINT;
            break;
        }
        if (step >= p.max_steps) {
            status = TRAJ_STEP_LIMIT;
            break;
        }
        if (step - dr.base >= 32ull) draws_fill(p, traj, step, lane, dr);
        const int src = (int)(step - dr.base);
        const float nlog = __shfl_sync(MBG_FULL, dr.nlog, src);
        const unsigned dy = __shfl_sync(MBG_FULL, dr.y, src);
        const unsigned dz = __shfl_sync(MBG_FULL, dr.z, src);
        const unsigned long long t1 = next_time(p, t, step, nlog, total);
        if (p.discrete) win_discrete(p, step, so, h, leader);
        else win_slice(acc, p, t, t1, so, h, leader);
        ++step;
        if (t1 >= p.max_time_fx) {
            t = p.max_time_fx;
            status = TRAJ_FINISHED;
            break;
        }
        if (p.redraw_period && step % p.redraw_period == 0ull) {  // a reference segment ends: no flip
            t = t1;
            continue;
        }
        // pick: register prefix (top level), L1 scan (N > 1024), leaf scan
        unsigned long long r = pick_target(dy, dz, total);
        const int tj = prefix_pick(pre, r);
        if (tj < 0 || tj >= top_count) { status = TRAJ_ERROR; break; }
        int g = tj;
        if (two_level) {
            const int gi = tj * 32 + (int)lane;
            const int jj = warp_pick(gi < G ? m.l1[gi] : 0ull, r, lane);
            if (jj < 0) { status = TRAJ_ERROR; break; }
            g = tj * 32 + jj;
        }
        int k = -1;
        const unsigned aw = m.act[g];
        if (!p.has_palette && __popc(aw) <= 4) {
            // few active nodes in the group (the usual case once most nodes have frozen): walk
            // them in node order; inactive nodes add nothing to the prefix
            const unsigned sw = m.st[g];
            unsigned rem = aw;
            while (rem) {
                const int b = __ffs(rem) - 1;
                rem &= rem - 1u;
                const int i = g * 32 + b;
                const unsigned long long v = __ldg(&p.nodes[i].up + ((sw >> b) & 1u));
                if (r < v) {
                    k = i;
                    break;
                }
                r -= v;
            }
            if (k < 0) { status = TRAJ_ERROR; break; }
        } else {
            const int i = g * 32 + (int)lane;
            const int jj = warp_pick(i < p.n ? current_rate<IDX>(p, i, m) : 0ull, r, lane);
            if (jj < 0) { status = TRAJ_ERROR; break; }
            k = g * 32 + jj;
        }
        // flip
        if (leader) m.st[k >> 5] ^= 1u << (k & 31);
        __syncwarp();
        // update the rates that read k, one reader per lane
        const int d0 = (int)__ldg(p.dep_off + k), d1 = (int)__ldg(p.dep_off + k + 1);
        bool out_touched = false;
        for (int qb = d0; qb < d1; qb += 32) {
            const int q = qb + (int)lane;
            unsigned long long delta = 0ull;
            int dn = 0;
            if (q < d1) {
                const unsigned e = __ldg(p.deps + q);
                dn = (int)(e >> 16);
                const int kd = (int)((e >> 8) & 0x7fu);
                const unsigned pos = e & 0xffu;
                const unsigned self = st_bit(m.st, dn);
                const unsigned self_old = pos == 0xffu ? self ^ 1u : self;
                // the reader's 32-byte record: rates, and for up to 4 regulators their ids and table
                const uint4* rec = reinterpret_cast<const uint4*>(p.lnodes + dn);
                const uint4 ra = __ldg(rec), rb = __ldg(rec + 1);
                const unsigned flags = rb.w >> 16;
                unsigned idx, idx_old;
                if (IDX) {
                    idx_old = m.idx[dn];
                    idx = pos == 0xffu ? idx_old : idx_old ^ (1u << pos);
                    if (pos != 0xffu) m.idx[dn] = idx;
                } else {
                    idx = flags == 0u ? warp_idx4(m.st, kd, rb.y, rb.z) : gather_regs(p, dn, load_head(p, dn), m.st);
                    idx_old = pos == 0xffu ? idx : idx ^ (1u << pos);
                }
                unsigned long long r_new, r_old;
                unsigned a_new, a_old;
                if (!(flags & kLanePalette)) {
                    const unsigned long long up = ((unsigned long long)ra.y << 32) | ra.x;
                    const unsigned long long down = ((unsigned long long)ra.w << 32) | ra.z;
                    a_new = flags == 0u ? (rb.x >> ((self << kd) | idx)) & 1u : table_bit(p, dn, kd, self, idx);
                    a_old = st_bit(m.act, dn);
                    r_new = a_new ? (self ? down : up) : 0ull;
                    r_old = a_old ? (self_old ? down : up) : 0ull;
                } else {
                    const NodeHead hd = load_head(p, dn);
                    r_new = palette_rate(p, hd, self, idx);
                    r_old = palette_rate(p, hd, self_old, idx_old);
                    a_new = r_new != 0ull;
                    a_old = r_old != 0ull;
                }
                if (a_new != a_old) atomicXor(m.act + (dn >> 5), 1u << (dn & 31));
                delta = r_new - r_old;
                if (delta != 0ull) {
                    if (two_level) atomicAdd(m.l1 + (dn >> 5), delta);
                    out_touched |= ((e >> 15) & 1u) != 0u;
                }
            }
            // broadcast each change into the register prefix
            unsigned mask = __ballot_sync(MBG_FULL, delta != 0ull);
            const int top_of = two_level ? (dn >> 10) : (dn >> 5);
            while (mask) {
                const int b = __ffs(mask) - 1;
                mask &= mask - 1u;
                const int tb = __shfl_sync(MBG_FULL, top_of, b);
                const unsigned long long d = __shfl_sync(MBG_FULL, delta, b);
                if ((int)lane >= tb) pre += d;
            }
        }
        total = __shfl_sync(MBG_FULL, pre, 31);
        __syncwarp();
        const short op = __ldg(p.out_pos + k);
        if (op >= 0) so ^= 1u << op;
        if (__any_sync(MBG_FULL, out_touched)) h = warp_entropy<IDX>(p, m, lane);
        t = t1;
        ++trans;
    }
    if (status == TRAJ_ERROR && leader) atomicOr(p.error_flag, (unsigned)DEV_ERR_PICK);
    if (!p.discrete && status != TRAJ_ERROR) win_end(acc, p, t, leader);
    c_trans += trans;
    c_steps += step + (status == TRAJ_FIXED_POINT ? 1 : 0);
    if (leader) record_end_scalar(p, j, status, t, trans, so);
    if (p.traj_state)
        for (int w = (int)lane; w < p.words; w += 32) p.traj_state[j * p.words + w] = m.st[w];
    if (status == TRAJ_FIXED_POINT) {
        unsigned slot = 0;
        if (leader) slot = atomicAdd(p.fp_count, 1u);
        slot = __shfl_sync(MBG_FULL, slot, 0);
        if (slot < p.fp_capacity) {
            for (int w = (int)lane; w < p.words; w += 32)
                p.fp_states[(unsigned long long)slot * p.words + w] = m.st[w];
        } else if (leader) {
            atomicOr(p.error_flag, (unsigned)DEV_ERR_FP_OVERFLOW);
        }
    }
    __syncwarp();
    return status;
}

__device__ __forceinline__ WarpSmem warp_smem_at(unsigned char* base, int n, bool cached_index) {
    WarpSmem m;
    const int L1 = warp_l1_smem(n), Wp = warp_words_padded(n);
    m.l1 = reinterpret_cast<unsigned long long*>(base);
    m.st = reinterpret_cast<unsigned*>(m.l1 + L1);
    m.act = m.st + Wp;
    m.idx = cached_index ? m.act + Wp : nullptr;
    return m;
}

struct WarpCounts {
    unsigned long long trans = 0, steps = 0;
    unsigned fin = 0, fix = 0, lim = 0, err = 0;

    __device__ __forceinline__ void add(unsigned char st) {
        fin += st == TRAJ_FINISHED;
        fix += st == TRAJ_FIXED_POINT;
        lim += st == TRAJ_STEP_LIMIT;
        err += st == TRAJ_ERROR;
    }
    // lane 0 only
    __device__ __forceinline__ void flush(unsigned long long* counters) {
        if (trans) atomicAdd(counters + CNT_TRANSITIONS, trans);
        if (steps) atomicAdd(counters + CNT_STEPS, steps);
        if (fin) atomicAdd(counters + CNT_FINISHED, (unsigned long long)fin);
        if (fix) atomicAdd(counters + CNT_FIXED, (unsigned long long)fix);
        if (lim) atomicAdd(counters + CNT_STEP_LIMIT, (unsigned long long)lim);
        if (err) atomicAdd(counters + CNT_ERROR, (unsigned long long)err);
        *this = WarpCounts();
    }
};

// Many independent instances (models, trajectory counts, seeds) in one persistent launch. Work
// items are numbered across instances by the prefix sums of their trajectory counts; a warp copies
// the SimParams of the instance it works on into its shared-memory slice and keeps it while
// consecutive work items stay in that instance.
__host__ __device__ __forceinline__ unsigned batch_params_bytes() { return (unsigned)((sizeof(SimParams) + 15) & ~15); }

template <bool IDX>
__device__ void sim_warp_batch_body(const BatchDesc& b, unsigned char* smem) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)warp * b.slice_bytes;
    SimParams* ps = reinterpret_cast<SimParams*>(base);
    unsigned char* ws = base + batch_params_bytes();
    const unsigned long long total = __ldg(b.prefix + b.n_inst);
    int cur = -1;
    WarpCounts c;
    for (;;) {
        unsigned long long j = 0;
        if (lane == 0) j = atomicAdd(b.work, 1ull);
        j = __shfl_sync(MBG_FULL, j, 0);
        if (j >= total) break;
        int lo = 0, hi = b.n_inst;  // prefix[lo] <= j < prefix[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(b.prefix + mid) <= j) lo = mid;
            else hi = mid;
        }
        if (lo != cur) {
            if (cur >= 0 && lane == 0) c.flush(ps->counters);
            __syncwarp();
            const unsigned* src = reinterpret_cast<const unsigned*>(b.params + lo);
            unsigned* dst = reinterpret_cast<unsigned*>(ps);
            for (int w = (int)lane; w < (int)(sizeof(SimParams) / 4); w += 32) dst[w] = __ldg(src + w);
            __syncwarp();
            cur = lo;
        }
        const WarpSmem m = warp_smem_at(ws, ps->n, IDX);
        c.add(warp_trajectory<IDX>(*ps, m, j - __ldg(b.prefix + lo), lane, c.trans, c.steps));
    }
    if (cur >= 0 && lane == 0) c.flush(ps->counters);
}

template <bool IDX>
__device__ void sim_warp_body(const SimParams& p, unsigned char* smem) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const WarpSmem m = warp_smem_at(smem + (size_t)warp * warp_smem_bytes(p.n, IDX), p.n, IDX);
    WarpCounts c;
    for (;;) {
        unsigned long long j = 0;
        if (lane == 0) j = atomicAdd(p.counters + CNT_WORK, 1ull);
        j = __shfl_sync(MBG_FULL, j, 0);
        if (j >= p.n_traj) break;
        c.add(warp_trajectory<IDX>(p, m, j, lane, c.trans, c.steps));
    }
    if (lane == 0) c.flush(p.counters);
}

}  // namespace mbg
