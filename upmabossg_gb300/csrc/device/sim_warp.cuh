// Warp-per-trajectory kernel for networks of hundreds to tens of thousands of nodes.
//
// One warp owns one trajectory. Its shared-memory slice holds the state words and two levels of
// exact 64-bit fixed-point rate sums: L1[g] over nodes 32g..32g+31 and L2[j] over groups
// 32j..32j+31 (N <= 32768). Per transition:
//   pick    warp inclusive scans (__shfl_up) over L2, then L1, then the 32 leaf rates of the
//           chosen group, each followed by a __ballot for the first prefix above the target;
//   flip    one shared-memory word;
//   update  the nodes that read the flipped node (CSR `deps`) are re-evaluated one per lane; the
//           exact difference of old and new rate goes into L1/L2 with shared atomics, so the
//           sums never drift and equal a from-scratch sum bit for bit.
// The reference instead recomputes all N rates into a thread-local array every step and scans
// it linearly (src/generator.cpp:124-144, src/jit_kernels/simulation.cu:9-21).
#pragma once

namespace mbg {

struct WarpSmem {
    unsigned long long* l1;
    unsigned long long* l2;
    unsigned* st;
};

__host__ __device__ __forceinline__ int warp_groups(int n) { return (n + 31) >> 5; }
__host__ __device__ __forceinline__ int warp_groups2(int n) { return (warp_groups(n) + 31) >> 5; }
// shared-memory bytes per warp: L1 + L2 (8 B each) + state words padded to 16 B
__host__ __device__ __forceinline__ unsigned warp_smem_bytes(int n) {
    int g = warp_groups(n), g2 = warp_groups2(n), w = (n + 31) >> 5;
    return (unsigned)(8 * (g + g2) + 16 * ((w + 3) >> 2));
}

__device__ __forceinline__ DevNode load_node(const SimParams& p, int i) {
    const uint4* q = reinterpret_cast<const uint4*>(p.nodes + i);
    uint4 a = __ldg(q), b = __ldg(q + 1);
    DevNode d;
    d.tab_off = a.x;
    d.reg_off = a.y;
    d.k = (unsigned short)(a.z & 0xffffu);
    d.kind = (unsigned short)(a.z >> 16);
    d.pal_off = a.w;
    d.up = ((unsigned long long)b.y << 32) | b.x;
    d.down = ((unsigned long long)b.w << 32) | b.z;
    return d;
}

__device__ __forceinline__ unsigned st_bit(const unsigned* st, int i) { return (st[i >> 5] >> (i & 31)) & 1u; }

// Regulator index of node `nd` in state `st`; `fm` gets the index bits that read node `k`.
__device__ __forceinline__ unsigned gather_regs(const SimParams& p, const DevNode& nd, const unsigned* st, int k,
                                                unsigned& fm) {
    unsigned idx = 0u, f = 0u;
    const unsigned short* rg = p.regs + nd.reg_off;
    for (int j = 0; j < nd.k; ++j) {
        int r = __ldg(rg + j);
        idx |= st_bit(st, r) << j;
        f |= (unsigned)(r == k) << j;
    }
    fm = f;
    return idx;
}

__device__ __forceinline__ unsigned long long table_rate(const SimParams& p, const DevNode& nd, unsigned self,
                                                         unsigned idx) {
    unsigned a = (self << nd.k) | idx;
    if (nd.kind == 0) {
        unsigned bit = (__ldg(p.tabs + nd.tab_off + (a >> 5)) >> (a & 31)) & 1u;
        return bit ? (self ? nd.down : nd.up) : 0ull;
    }
    return __ldg(p.palette + nd.pal_off + __ldg(p.pidx + nd.tab_off + a));
}

__device__ __forceinline__ unsigned long long node_rate(const SimParams& p, int i, const unsigned* st) {
    DevNode nd = load_node(p, i);
    unsigned fm;
    unsigned idx = gather_regs(p, nd, st, -1, fm);
    return table_rate(p, nd, st_bit(st, i), idx);
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
        unsigned long long o = __shfl_up_sync(MBG_FULL, v, d);
        if (lane >= (unsigned)d) v += o;
    }
    return v;
}

// Chooses the lane whose inclusive prefix first exceeds r; r becomes relative to that lane.
// Returns -1 if no lane qualifies (inconsistent sums).
__device__ __forceinline__ int warp_pick(unsigned long long v, unsigned long long& r, unsigned lane) {
    unsigned long long inc = warp_scan_u64(v, lane);
    unsigned b = __ballot_sync(MBG_FULL, inc > r);
    if (b == 0u) return -1;
    int j = __ffs(b) - 1;
    unsigned long long excl = __shfl_sync(MBG_FULL, inc - v, j);
    r -= excl;
    return j;
}

// Transition entropy of the current state, -sum p log2 p over the output nodes, one output node
// per lane (generator.cpp:146-175). The warp path requires n_out <= 32.
__device__ __forceinline__ float warp_entropy(const SimParams& p, const unsigned* st, unsigned lane) {
    unsigned long long r = 0ull;
    if ((int)lane < p.n_out) r = node_rate(p, __ldg(p.out_nodes + lane), st);
    const unsigned long long R = warp_sum_u64(r);
    if (R == 0ull) return 0.f;
    const float pr = (float)r / (float)R;
    const float term = pr > 0.f ? pr * __log2f(pr) : 0.f;
    const float h = -warp_sum_f32(term);
    return h > 0.f ? h : 0.f;
}

__device__ __forceinline__ unsigned warp_out_index(const SimParams& p, const unsigned* st, unsigned lane) {
    unsigned b = 0u;
    if ((int)lane < p.n_out) b = st_bit(st, __ldg(p.out_nodes + lane));
    return __ballot_sync(MBG_FULL, b != 0u);
}

// Fills L1, L2 from scratch; returns the total rate.
__device__ __forceinline__ unsigned long long warp_build_sums(const SimParams& p, WarpSmem m, unsigned lane) {
    const int G = warp_groups(p.n), G2 = warp_groups2(p.n);
    for (int g = 0; g < G; ++g) {
        int i = g * 32 + (int)lane;
        unsigned long long v = i < p.n ? node_rate(p, i, m.st) : 0ull;
        v = warp_sum_u64(v);
        if (lane == 0) m.l1[g] = v;
    }
    __syncwarp();
    for (int j = (int)lane; j < G2; j += 32) {
        unsigned long long v = 0ull;
        for (int g = 32 * j; g < G && g < 32 * j + 32; ++g) v += m.l1[g];
        m.l2[j] = v;
    }
    __syncwarp();
    unsigned long long tot = 0ull;
    for (int j = (int)lane; j < G2; j += 32) tot += m.l2[j];
    return warp_sum_u64(tot);
}

__device__ __forceinline__ void warp_init_state(const SimParams& p, unsigned long long traj, unsigned* st,
                                                unsigned lane) {
    const int W = p.words;
    for (int w = (int)lane; w < W; w += 32) {
        unsigned word = 0u;
        for (int b = 0; b < 8; ++b) {
            int blk = w * 8 + b;
            if (4 * blk >= p.n) break;
            u32x4 d = philox_init(p.seed, traj, (unsigned)blk);
            unsigned v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                int i = 4 * blk + c;
                if (i < p.n && (v[c] >> 8) < __ldg(p.istate_thr + i)) word |= 1u << (i & 31);
            }
        }
        st[w] = word;
    }
    __syncwarp();
}

// One trajectory, run by the whole warp. Returns the end status; counts go to the references.
__device__ unsigned char warp_trajectory(const SimParams& p, WarpSmem m, unsigned long long j, unsigned lane,
                                         unsigned long long& c_trans, unsigned long long& c_steps) {
    const bool leader = lane == 0u;
    const int G2 = warp_groups2(p.n);
    const unsigned long long traj = p.traj_base + j;
    warp_init_state(p, traj, m.st, lane);
    unsigned long long total = warp_build_sums(p, m, lane);
    unsigned so = warp_out_index(p, m.st, lane);
    float h = warp_entropy(p, m.st, lane);
    WindowAcc acc;
    win_begin(acc, p, so);
    double t = 0.0;
    unsigned long long step = 0;
    unsigned trans = 0;
    unsigned char status = TRAJ_CONTINUE;
    for (;;) {
        if (total == 0ull) {
            if (p.discrete) win_discrete(p, step, so, 0.f, leader);
            else win_slice(acc, p, t, p.max_time, so, 0.f, leader);
            t = p.max_time;
            status = TRAJ_FIXED_POINT;
            break;
        }
        if (step >= p.max_steps) {
            status = TRAJ_STEP_LIMIT;
            break;
        }
        const u32x4 d = philox_step(p.seed, traj, step);
        const double t1 = next_time(p, t, step, d.x, total);
        if (p.discrete) win_discrete(p, step, so, h, leader);
        else win_slice(acc, p, t, t1, so, h, leader);
        ++step;
        if (t1 >= p.max_time) {
            t = p.max_time;
            status = TRAJ_FINISHED;
            break;
        }
        // pick
        unsigned long long r = pick_target(d.y, d.z, total);
        int base = 0;
        if (G2 > 1) {
            unsigned long long v = (int)lane < G2 ? m.l2[lane] : 0ull;
            int jj = warp_pick(v, r, lane);
            if (jj < 0) { status = TRAJ_ERROR; break; }
            base = jj * 32;
        }
        int g;
        {
            int gi = base + (int)lane;
            unsigned long long v = gi < warp_groups(p.n) ? m.l1[gi] : 0ull;
            int jj = warp_pick(v, r, lane);
            if (jj < 0) { status = TRAJ_ERROR; break; }
            g = base + jj;
        }
        int k;
        {
            int i = g * 32 + (int)lane;
            unsigned long long v = i < p.n ? node_rate(p, i, m.st) : 0ull;
            int jj = warp_pick(v, r, lane);
            if (jj < 0) { status = TRAJ_ERROR; break; }
            k = g * 32 + jj;
        }
        // flip
        if (leader) m.st[k >> 5] ^= 1u << (k & 31);
        __syncwarp();
        // update the rates that read k
        const int d0 = (int)__ldg(p.dep_off + k), d1 = (int)__ldg(p.dep_off + k + 1);
        unsigned long long dsum = 0ull;
        bool out_touched = false;
        for (int q = d0 + (int)lane; q < d1; q += 32) {
            const int dn = __ldg(p.deps + q);
            const DevNode nd = load_node(p, dn);
            unsigned fm;
            const unsigned idx = gather_regs(p, nd, m.st, k, fm);
            const unsigned self = st_bit(m.st, dn);
            const unsigned self_old = dn == k ? self ^ 1u : self;
            const unsigned long long delta = table_rate(p, nd, self, idx) - table_rate(p, nd, self_old, idx ^ fm);
            if (delta != 0ull) {
                atomicAdd(m.l1 + (dn >> 5), delta);
                if (G2 > 1) atomicAdd(m.l2 + (dn >> 10), delta);
                dsum += delta;
                out_touched |= __ldg(p.out_pos + dn) >= 0;
            }
        }
        total += warp_sum_u64(dsum);
        __syncwarp();
        const short op = __ldg(p.out_pos + k);
        if (op >= 0) so ^= 1u << op;
        if (__any_sync(MBG_FULL, out_touched)) h = warp_entropy(p, m.st, lane);
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

__device__ void sim_warp_body(const SimParams& p, unsigned char* smem) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int G = warp_groups(p.n), G2 = warp_groups2(p.n);
    unsigned char* base = smem + (size_t)warp * warp_smem_bytes(p.n);
    WarpSmem m;
    m.l1 = reinterpret_cast<unsigned long long*>(base);
    m.l2 = m.l1 + G;
    m.st = reinterpret_cast<unsigned*>(m.l2 + G2);
    unsigned long long c_trans = 0, c_steps = 0;
    unsigned c_fin = 0, c_fix = 0, c_lim = 0, c_err = 0;
    for (;;) {
        unsigned long long j = 0;
        if (lane == 0) j = atomicAdd(p.counters + CNT_WORK, 1ull);
        j = __shfl_sync(MBG_FULL, j, 0);
        if (j >= p.n_traj) break;
        unsigned char st = warp_trajectory(p, m, j, lane, c_trans, c_steps);
        c_fin += st == TRAJ_FINISHED;
        c_fix += st == TRAJ_FIXED_POINT;
        c_lim += st == TRAJ_STEP_LIMIT;
        c_err += st == TRAJ_ERROR;
    }
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
