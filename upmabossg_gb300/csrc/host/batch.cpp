// Batched parameter sweeps: every instance's model image and results live in a few arenas; the
// instances are grouped by model size into classes, each class runs in one persistent launch of
// the lane or the warp layout with its own launch shape, and the clearing, the class launches, the
// fixed-point aggregation and the counter read-back are captured once into a CUDA graph.
// The reference has no batching: a sweep is one CLI run per instance (src/main.cpp:101-169),
// each with its own NVRTC compilation (src/kernel_compiler.cpp:61-164) and batch loop
// (src/simulation_runner.cu:54-180).
#include "batch.hpp"

#include <algorithm>
#include <cstring>

#include "../device/kernels.h"
#include "devmem.hpp"
#include "parallel.hpp"

namespace mbg {

namespace {

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

struct Layout {
    size_t size = 0;
    size_t add(size_t bytes) {
        size_t off = (size + 255) & ~(size_t)255;
        size = off + (bytes ? bytes : 1);
        return off;
    }
};

// Device blocks come from the process-wide block cache (devmem.hpp): a sweep that creates one batch
// after another of the same shape reuses the blocks instead of allocating and freeing them.
void* dmalloc(size_t bytes, std::vector<void*>& owned) {
    void* p = dev_alloc(bytes, "batch arena");
    owned.push_back(p);
    return p;
}

constexpr size_t kSmallPerInst = 96;  // 8 u64 counters, error word, unique fixed points
// Size classes by 32-node groups, a power of two apart: up to 32, 64, ..., 4096 nodes, larger.
// (Classes 1.4x apart, which size a class's shared-memory rows closer to each member, measured
// 2% slower on the 256-instance sweep: 167 against 170 points/s.)
constexpr int kClasses = 8;
constexpr size_t kSmemLimit = 227 * 1024;

}  // namespace

int batch_size_class(int n) {
    const int g = (n + 31) / 32;  // 32-node groups
    int c = 0;
    while ((1 << c) < g && c < kClasses - 1) ++c;
    return c;
}

Batch::~Batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    for (cudaEvent_t e : {ev0, ev1})
        if (e) cudaEventDestroy(e);
    for (Class& k : classes) {
        for (cudaEvent_t e : {k.e0, k.e1, k.join})
            if (e) cudaEventDestroy(e);
        if (k.stream) cudaStreamDestroy(k.stream);
    }
    if (fork) cudaEventDestroy(fork);
    // the blocks go back to the cache: nothing of this batch may still run on them
    cudaDeviceSynchronize();
    for (Class& k : classes) dev_free(k.lane_buf);
    pinned_free(small_host);
    for (void* p : owned) dev_free(p);
}

void Batch::create(const std::vector<const CompiledModel*>& models, const std::vector<uint64_t>& n_traj,
                   const std::vector<uint64_t>& seeds, const mbg_batch_opts& o) {
    if (models.empty()) throw ArgError("empty batch");
    if (o.block_size && (o.block_size % 32 != 0 || o.block_size > 256))
        throw ArgError("block_size must be a multiple of 32, at most 256");
    if (o.layout != 0 && o.layout != MBG_LAYOUT_LANE && o.layout != MBG_LAYOUT_WARP &&
        o.layout != MBG_LAYOUT_LANE_GLOBAL)
        throw ArgError("batch layout must be 0 (auto), MBG_LAYOUT_LANE, MBG_LAYOUT_LANE_GLOBAL or MBG_LAYOUT_WARP");
    if (o.lane_variant < 0 || o.lane_variant > 2) throw ArgError("lane_variant must be 0, 1 or 2");
    opts = o;
    for (size_t i = 0; i < models.size(); ++i)  // argument checks come before any device call
        check_model_limits(*models[i], n_traj.empty() || n_traj[i] == 0 ? models[i]->sample_count : n_traj[i]);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw CudaError("no CUDA device available");
    }
    device = o.device;
    if (device < 0 || device >= ndev) throw ArgError("device ordinal out of range");
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");

    const size_t n = models.size();
    inst.resize(n);
    // size classes; the class-ordered arrays (params, fixed-point slots) list class 0's members
    // first, then class 1's, ...
    std::vector<Class> all(kClasses);
    for (size_t i = 0; i < n; ++i) {
        Inst& x = inst[i];
        const CompiledModel& cm = *models[i];
        x.n_traj = n_traj.empty() || n_traj[i] == 0 ? cm.sample_count : n_traj[i];
        x.seed = seeds.empty() ? cm.seed : seeds[i];
        if (cm.n_out > 32) throw ModelError("batched instances support at most 32 outputs");
        Class& k = all[batch_size_class(cm.n)];
        k.members.push_back((int)i);
        k.max_n = std::max(k.max_n, cm.n);
        for (const auto& nd : cm.nodes) k.full |= nd.kind == NODE_PALETTE;
        k.full |= cm.max_k > 12;
        k.traj += x.n_traj;
    }
    // every instance's model copy and device layout (host work, independent per instance)
    std::vector<DeviceLayout> dls(n);
    parallel_items<int>((int)n, 64, [&](int i, int&) {
        inst[i].cm = *models[i];
        dls[i] = layout_model(inst[i].cm);
        check_layout(inst[i].cm, dls[i]);
    });
    for (Class& k : all)
        if (!k.members.empty()) classes.push_back(std::move(k));
    std::vector<int> order;  // class order -> instance
    for (size_t c = 0; c < classes.size(); ++c) {
        classes[c].first = order.size();
        for (int i : classes[c].members) {
            inst[i].cls = (int)c;
            order.push_back(i);
        }
    }

    Layout ml, rl, pl, fl;
    struct Off {
        size_t nodes, lnodes, lwide, regs, tabs, pidx, palette, dep_off, deps, out_nodes, out_pos, istate;
        size_t hist, th, fin, fp_count, slot_cnt, rep, fp_states, out_states, out_cnt;
    };
    std::vector<Off> off(n);
    for (size_t i = 0; i < n; ++i) {
        Inst& x = inst[i];
        const CompiledModel& cm = x.cm;
        total_traj += x.n_traj;
        const DeviceLayout& d = dls[i];
        Off& f = off[i];
        f.nodes = ml.add(d.nodes.size() * sizeof(DevNode));
        f.lnodes = ml.add(d.lnodes.size() * sizeof(LaneNode));
        f.lwide = ml.add(d.lwide.size() * sizeof(LaneWide));
        f.regs = ml.add(d.regs.size() * 2);
        f.tabs = ml.add(d.tabs.size() * 4);
        f.pidx = ml.add(d.pidx.size());
        f.palette = ml.add(d.palette.size() * 8);
        f.dep_off = ml.add(d.dep_off.size() * 4);
        f.deps = ml.add(d.deps.size() * 4);
        f.out_nodes = ml.add(d.out_nodes.size() * 2);
        f.out_pos = ml.add(d.out_pos.size() * 2);
        f.istate = ml.add(d.istate_thr.size() * 4);
        const uint64_t S = 1ull << cm.n_out;
        const uint32_t cap = (uint32_t)x.n_traj;
        x.fp.n_slots = fp_slot_count(cap);
        f.hist = rl.add(cm.windows * S * 8);
        f.th = rl.add(cm.windows * 8);
        f.fin = rl.add(S * 4);
        f.fp_count = rl.add(4);
        f.slot_cnt = rl.add((size_t)x.fp.n_slots * 4);
        f.rep = pl.add((size_t)x.fp.n_slots * 4);
        f.fp_states = fl.add((size_t)cap * cm.words * 4);
        f.out_states = fl.add((size_t)cap * cm.words * 4);
        f.out_cnt = fl.add((size_t)cap * 4);
    }
    small_bytes = n * kSmallPerInst + 8 * classes.size();  // + one work counter per class
    const size_t small_off = rl.add(small_bytes);

    // model arena: one staging buffer, one copy
    char* model_arena = static_cast<char*>(dmalloc(ml.size, owned));
    std::vector<char> stage(ml.size, 0);
    auto put = [&](size_t o2, const void* src, size_t bytes) {
        if (bytes) std::memcpy(stage.data() + o2, src, bytes);
    };
    for (size_t i = 0; i < n; ++i) {
        const DeviceLayout& d = dls[i];
        const Off& f = off[i];
        put(f.nodes, d.nodes.data(), d.nodes.size() * sizeof(DevNode));
        put(f.lnodes, d.lnodes.data(), d.lnodes.size() * sizeof(LaneNode));
        put(f.lwide, d.lwide.data(), d.lwide.size() * sizeof(LaneWide));
        put(f.regs, d.regs.data(), d.regs.size() * 2);
        put(f.tabs, d.tabs.data(), d.tabs.size() * 4);
        put(f.pidx, d.pidx.data(), d.pidx.size());
        put(f.palette, d.palette.data(), d.palette.size() * 8);
        put(f.dep_off, d.dep_off.data(), d.dep_off.size() * 4);
        put(f.deps, d.deps.data(), d.deps.size() * 4);
        put(f.out_nodes, d.out_nodes.data(), d.out_nodes.size() * 2);
        put(f.out_pos, d.out_pos.data(), d.out_pos.size() * 2);
        put(f.istate, d.istate_thr.data(), d.istate_thr.size() * 4);
    }
    ck(cudaMemcpy(model_arena, stage.data(), ml.size, cudaMemcpyHostToDevice), "cudaMemcpy H2D");

    char* res = static_cast<char*>(dmalloc(rl.size, owned));
    result_arena = res;
    result_bytes = rl.size;
    char* rep = static_cast<char*>(dmalloc(pl.size, owned));
    rep_arena = rep;
    rep_bytes = pl.size;
    char* fpa = static_cast<char*>(dmalloc(fl.size, owned));
    small_dev = res + small_off;
    small_host = static_cast<char*>(pinned_alloc(small_bytes));

    std::vector<SimParams> prms(n);
    std::vector<FpSlots> fps(n);
    for (size_t pos = 0; pos < n; ++pos) {
        const size_t i = (size_t)order[pos];
        Inst& x = inst[i];
        const Off& f = off[i];
        SimParams& p = x.prm;
        std::memset(&p, 0, sizeof p);
        p.nodes = reinterpret_cast<const DevNode*>(model_arena + f.nodes);
        p.lnodes = reinterpret_cast<const LaneNode*>(model_arena + f.lnodes);
        p.lwide = reinterpret_cast<const LaneWide*>(model_arena + f.lwide);
        p.regs = reinterpret_cast<const unsigned short*>(model_arena + f.regs);
        p.tabs = reinterpret_cast<const unsigned*>(model_arena + f.tabs);
        p.pidx = reinterpret_cast<const unsigned char*>(model_arena + f.pidx);
        p.palette = reinterpret_cast<const unsigned long long*>(model_arena + f.palette);
        p.dep_off = reinterpret_cast<const unsigned*>(model_arena + f.dep_off);
        p.deps = reinterpret_cast<const unsigned*>(model_arena + f.deps);
        p.out_nodes = reinterpret_cast<const unsigned short*>(model_arena + f.out_nodes);
        p.out_pos = reinterpret_cast<const short*>(model_arena + f.out_pos);
        p.istate_thr = reinterpret_cast<const unsigned*>(model_arena + f.istate);
        set_model_constants(p, x.cm);
        p.max_steps = o.max_steps ? o.max_steps : 0xFFFFFFFFu;
        p.seed = x.seed;
        p.n_traj = x.n_traj;
        p.traj_base = 0;
        p.hist = reinterpret_cast<unsigned long long*>(res + f.hist);
        p.th_hist = reinterpret_cast<unsigned long long*>(res + f.th);
        p.final_hist = reinterpret_cast<unsigned*>(res + f.fin);
        p.fp_count = reinterpret_cast<unsigned*>(res + f.fp_count);
        p.fp_capacity = (unsigned)x.n_traj;
        p.fp_states = reinterpret_cast<unsigned*>(fpa + f.fp_states);
        x.small_off = i * kSmallPerInst;
        p.counters = reinterpret_cast<unsigned long long*>(small_dev + x.small_off);
        p.error_flag = reinterpret_cast<unsigned*>(small_dev + x.small_off + 8 * CNT_COUNT);
        x.fp.slot_rep = reinterpret_cast<unsigned*>(rep + f.rep);
        x.fp.slot_cnt = reinterpret_cast<unsigned*>(res + f.slot_cnt);
        x.fp.out_states = reinterpret_cast<unsigned*>(fpa + f.out_states);
        x.fp.out_cnt = reinterpret_cast<unsigned*>(fpa + f.out_cnt);
        x.fp.n_unique = reinterpret_cast<unsigned*>(small_dev + x.small_off + 8 * CNT_COUNT + 4);
        prms[pos] = p;
        fps[pos] = x.fp;
    }
    d_params = static_cast<SimParams*>(dmalloc(n * sizeof(SimParams), owned));
    d_fps = static_cast<FpSlots*>(dmalloc(n * sizeof(FpSlots), owned));
    ck(cudaMemcpy(d_params, prms.data(), n * sizeof(SimParams), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ck(cudaMemcpy(d_fps, fps.data(), n * sizeof(FpSlots), cudaMemcpyHostToDevice), "cudaMemcpy H2D");

    // per class: trajectory prefixes over its members, and a pilot of about 256k trajectories
    // (every member keeps at least one) for timing launch shapes
    for (size_t c = 0; c < classes.size(); ++c) {
        Class& k = classes[c];
        const size_t m = k.members.size();
        std::vector<unsigned long long> prefix(m + 1, 0), pilot(m + 1, 0), pilot4(m + 1, 0);
        const double scale = std::min(1.0, 262144.0 / (double)k.traj);
        const double scale4 = std::min(1.0, 4.0 * 262144.0 / (double)k.traj);
        for (size_t q = 0; q < m; ++q) {
            const uint64_t nt = inst[k.members[q]].n_traj;
            prefix[q + 1] = prefix[q] + nt;
            pilot[q + 1] = pilot[q] + std::max<uint64_t>(1, (uint64_t)((double)nt * scale));
            pilot4[q + 1] = pilot4[q] + std::max<uint64_t>(1, (uint64_t)((double)nt * scale4));
        }
        auto* dp = static_cast<unsigned long long*>(dmalloc((m + 1) * 8, owned));
        auto* dq = static_cast<unsigned long long*>(dmalloc((m + 1) * 8, owned));
        auto* dq4 = static_cast<unsigned long long*>(dmalloc((m + 1) * 8, owned));
        ck(cudaMemcpy(dp, prefix.data(), (m + 1) * 8, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        ck(cudaMemcpy(dq, pilot.data(), (m + 1) * 8, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        ck(cudaMemcpy(dq4, pilot4.data(), (m + 1) * 8, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        k.has_long = pilot4[m] > pilot[m];
        k.desc.params = d_params + k.first;
        k.desc.prefix = dp;
        k.desc.n_inst = (int)m;
        k.desc.work = reinterpret_cast<unsigned long long*>(small_dev + n * kSmallPerInst + 8 * c);
        k.desc.rows = sim_lane_rows(k.max_n);
        k.pilot = k.desc;
        k.pilot.prefix = dq;
        k.pilot_long = k.desc;
        k.pilot_long.prefix = dq4;
        ck(cudaEventCreate(&k.e0), "cudaEventCreate");
        ck(cudaEventCreate(&k.e1), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&k.join, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaStreamCreateWithFlags(&k.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    }

    ck(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    for (cudaEvent_t* e : {&ev0, &ev1}) ck(cudaEventCreate(e), "cudaEventCreate");
    // default shapes (the autotuner replaces them on the first run): the lane layout at 128
    // threads per block where its shared memory fits, else the warp layout
    for (size_t c = 0; c < classes.size(); ++c) {
        Class& k = classes[c];
        const int blk = o.block_size > 0 ? o.block_size : 128;
        const bool lane_fits = sim_lane_smem(k.max_n, blk) <= kSmemLimit;
        const int lay = o.layout ? o.layout : (lane_fits ? MBG_LAYOUT_LANE : MBG_LAYOUT_WARP);
        if (lay == MBG_LAYOUT_LANE && !lane_fits)
            throw ModelError("largest instance of a size class too large for the batched lane layout");
        const int variant =
            lay == MBG_LAYOUT_WARP ? ((size_t)(blk / 32) * sim_warp_batch_slice_bytes(k.max_n, true) <= 100 * 1024)
            : lay == MBG_LAYOUT_LANE ? o.lane_variant : 0;
        configure((int)c, lay, blk, variant);
    }
    build_graph();
}

void Batch::configure(int c, int lay, int blk, int variant) {
    Class& k = classes[c];
    if (variant < 0 || variant > 2 || (lay != MBG_LAYOUT_LANE && variant > 1))
        throw ArgError("batched lane variant must be 0, 1 or 2");
    int bps = 0;
    size_t sm = 0;
    size_t row_bytes = 0;  // per block, in global memory
    if (lay == MBG_LAYOUT_LANE && variant == 2) {
        sm = sim_lane_split_smem(k.max_n, blk);
        if (sm > kSmemLimit) throw ModelError("largest instance of a size class too large for the batched lane layout");
        ck(sim_lane_batch_split_configure(k.full, sm, blk, &bps), "batched lane kernel occupancy");
        row_bytes = (size_t)sim_lane_rows(k.max_n) * 4 * (size_t)blk;  // the active words
    } else if (lay == MBG_LAYOUT_LANE) {
        sm = sim_lane_smem(k.max_n, blk);
        if (sm > kSmemLimit) throw ModelError("largest instance of a size class too large for the batched lane layout");
        ck(sim_lane_batch_configure(variant == 1, k.full, sm, blk, &bps), "batched lane kernel occupancy");
    } else if (lay == MBG_LAYOUT_LANE_GLOBAL) {
        variant = 0;  // per-lane reader update only
        ck(sim_lane_batch_global_configure(k.full, blk, &bps), "batched global-row lane kernel occupancy");
        row_bytes = sim_lane_smem(k.max_n, blk);  // every row
    } else {
        const unsigned slice = sim_warp_batch_slice_bytes(k.max_n, variant != 0);
        sm = (size_t)(blk / 32) * slice;
        if (sm > kSmemLimit) throw ModelError("largest instance of a size class too large for the batched warp layout");
        ck(sim_warp_batch_configure(variant != 0, sm, blk, &bps), "batched warp kernel occupancy");
        // every work description a launch of this shape may run (the long pilot included: the
        // autotuner re-times the closest shapes on it)
        k.desc.slice_bytes = k.pilot.slice_bytes = k.pilot_long.slice_bytes = slice;
    }
    if (row_bytes) {
        if (bps < 1) throw CudaError("batched kernel cannot be resident with this block size");
        if (opts.blocks_per_sm > 0) bps = std::min(bps, (int)opts.blocks_per_sm);
        // one share of rows per resident block, 256-byte aligned
        const size_t block_bytes = (row_bytes + 255) & ~(size_t)255;
        const size_t need = block_bytes * (size_t)sms * (size_t)bps;
        if (need > k.lane_buf_bytes) {
            if (k.lane_buf) {
                cudaDeviceSynchronize();  // a pilot may still run on the old rows
                dev_free(k.lane_buf);
            }
            k.lane_buf = nullptr;
            k.lane_buf_bytes = 0;
            k.lane_buf = dev_alloc(need, "batch lane rows");
            k.lane_buf_bytes = need;
        }
        for (BatchDesc* d : {&k.desc, &k.pilot, &k.pilot_long}) {
            d->lane_state = static_cast<unsigned char*>(k.lane_buf);
            d->lane_block_bytes = block_bytes;
        }
    }
    if (bps < 1) throw CudaError("batched kernel cannot be resident with this block size");
    if (opts.blocks_per_sm > 0) bps = std::min(bps, (int)opts.blocks_per_sm);
    k.layout = lay;
    k.block = blk;
    k.variant = variant;
    k.smem = sm;
    k.grid = sms * bps;
}

cudaError_t Batch::launch_class(const Class& k, const BatchDesc& d, cudaStream_t s) const {
    if (k.layout == MBG_LAYOUT_LANE && k.variant == 2)
        return launch_sim_lane_batch_split(d, k.full, k.grid, k.block, k.smem, s);
    if (k.layout == MBG_LAYOUT_LANE)
        return launch_sim_lane_batch(d, k.variant == 1, k.full, k.grid, k.block, k.smem, s);
    if (k.layout == MBG_LAYOUT_LANE_GLOBAL) return launch_sim_lane_batch_global(d, k.full, k.grid, k.block, s);
    return launch_sim_warp_batch(d, k.variant, k.grid, k.block, k.smem, s);
}

void Batch::build_graph() {
    if (exec) {
        cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
    if (graph) {
        cudaGraphDestroy(graph);
        graph = nullptr;
    }
    cudaStream_t s = capture_stream;
    apply_limits();
    ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t e = cudaMemsetAsync(result_arena, 0, result_bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(rep_arena, 0xFF, rep_bytes, s);
    // one launch per size class, each on its own branch of the graph so that a class starts on the
    // SMs the previous one's last blocks leave instead of waiting for its whole tail; the largest
    // class first. Each launch is bracketed by external event-record nodes so that its kernel time
    // can be read after every replay.
    if (e == cudaSuccess) e = cudaEventRecord(fork, s);
    for (size_t ci = classes.size(); ci-- > 0;) {
        const Class& k = classes[ci];
        if (e == cudaSuccess) e = cudaStreamWaitEvent(k.stream, fork, 0);
        if (e == cudaSuccess) e = cudaEventRecordWithFlags(k.e0, k.stream, cudaEventRecordExternal);
        if (e == cudaSuccess) e = launch_class(k, k.desc, k.stream);
        if (e == cudaSuccess) e = cudaEventRecordWithFlags(k.e1, k.stream, cudaEventRecordExternal);
        if (e == cudaSuccess) e = cudaEventRecord(k.join, k.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, k.join, 0);
    }
    if (e == cudaSuccess) e = launch_fp_aggregate_batch(d_params, d_fps, (int)inst.size(), 8, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(small_host, small_dev, small_bytes, cudaMemcpyDeviceToHost, s);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    ck(e, "capturing the batch graph");
    ck(e2, "cudaStreamEndCapture");
    graph = g;
    ck(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
}

void Batch::autotune() {
    // Per size class, every shape (lane layout: threads per block x reader-update variant; warp
    // layout: threads per block x regulator-index cache) runs the class's pilot trajectories twice
    // and the second run's kernel time decides. Pilot runs write into the result buffers, which
    // the graph clears before every real run; a fixed-point buffer that fills up during the pilots
    // only sets an error bit in those buffers.
    const bool log = std::getenv("MBG_AUTOTUNE_LOG") != nullptr;
    cudaStream_t s = capture_stream;
    for (size_t c = 0; c < classes.size(); ++c) {
        Class& k = classes[c];
        k.timings.clear();
        double best = -1;
        int best_lay = k.layout, best_blk = k.block;
        int best_var = k.variant;
        // global rows only where shared memory holds fewer than 512 of a class's trajectories
        // per SM (rows over 454 B: above 1184 nodes); below that the shared-memory lane layout is
        // faster
        const bool try_global = opts.layout == MBG_LAYOUT_LANE_GLOBAL || sim_lane_smem(k.max_n, 512) > kSmemLimit;
        // the active words in global memory (lane variant 2) only where the shared-memory rows hold
        // fewer than three blocks of 256 per SM (the register limit of the batched lane kernels)
        const bool try_split = sim_lane_smem(k.max_n, 768) > kSmemLimit;
        for (int lay : {MBG_LAYOUT_LANE, MBG_LAYOUT_WARP, MBG_LAYOUT_LANE_GLOBAL}) {
            if (opts.layout && lay != opts.layout) continue;
            if (lay == MBG_LAYOUT_LANE_GLOBAL && !try_global) continue;
            for (int blk : {64, 128, 256}) {
                if (opts.block_size > 0 && blk != opts.block_size) continue;
                for (int var = 0; var < 3; ++var) {
                    if (lay == MBG_LAYOUT_LANE_GLOBAL && (var || blk == 64)) continue;
                    if (lay == MBG_LAYOUT_WARP && var == 2) continue;
                    if (lay == MBG_LAYOUT_LANE && var < 2 && sim_lane_smem(k.max_n, blk) > kSmemLimit) continue;
                    if (lay == MBG_LAYOUT_LANE && var == 2 &&
                        (!try_split || blk == 64 || sim_lane_split_smem(k.max_n, blk) > kSmemLimit))
                        continue;
                    if (lay == MBG_LAYOUT_WARP &&
                        (size_t)(blk / 32) * sim_warp_batch_slice_bytes(k.max_n, var != 0) > 100 * 1024)
                        continue;
                    configure((int)c, lay, blk, var);
                    float ms = 0.f;
                    for (int rep = 0; rep < 2; ++rep) {
                        ck(cudaMemsetAsync(k.desc.work, 0, 8, s), "cudaMemsetAsync");
                        ck(cudaEventRecord(ev0, s), "cudaEventRecord");
                        ck(launch_class(k, k.pilot, s), "autotune launch");
                        ck(cudaEventRecord(ev1, s), "cudaEventRecord");
                        ck(cudaStreamSynchronize(s), "autotune run");
                        ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
                    }
                    k.timings.push_back(mbg_batch_class_timing{lay, blk, var, 0, (double)ms});
                    if (log)
                        std::fprintf(stderr, "mbg batch autotune: class max_n=%d layout=%d block=%d variant=%d kernel_ms=%.3f\n",
                                     k.max_n, lay, blk, var, ms);
                    if (best < 0 || ms < best) {
                        best = ms;
                        best_lay = lay;
                        best_blk = blk;
                        best_var = var;
                    }
                }
            }
        }
        // a short pilot starts every lane's first trajectory together; the closest shapes are
        // timed again on a pilot four times longer, nearer the steady state of a full run
        if (k.has_long && k.timings.size() > 1) {
            std::vector<mbg_batch_class_timing> order = k.timings;
            std::sort(order.begin(), order.end(),
                      [](const mbg_batch_class_timing& a, const mbg_batch_class_timing& b) { return a.kernel_ms < b.kernel_ms; });
            // the three fastest within 15%, and the fastest of every (layout, variant) within 30%:
            // a short pilot can misrank the reader-update variants
            std::vector<size_t> pick;
            for (size_t i = 0; i < order.size(); ++i) {
                bool first_of_kind = true;
                for (size_t j = 0; j < i; ++j)
                    if (order[j].layout == order[i].layout && order[j].variant == order[i].variant) first_of_kind = false;
                if ((i < 3 && order[i].kernel_ms <= 1.15 * order[0].kernel_ms) ||
                    (first_of_kind && order[i].kernel_ms <= 1.3 * order[0].kernel_ms))
                    pick.push_back(i);
            }
            best = -1;
            for (size_t i : pick) {
                const mbg_batch_class_timing& t = order[i];
                configure((int)c, t.layout, t.block_size, t.variant);
                float ms = 0.f;
                ck(cudaMemsetAsync(k.desc.work, 0, 8, s), "cudaMemsetAsync");
                ck(cudaEventRecord(ev0, s), "cudaEventRecord");
                ck(launch_class(k, k.pilot_long, s), "autotune launch");
                ck(cudaEventRecord(ev1, s), "cudaEventRecord");
                ck(cudaStreamSynchronize(s), "autotune run");
                ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
                if (log)
                    std::fprintf(stderr, "mbg batch autotune: class max_n=%d long pilot layout=%d block=%d variant=%d kernel_ms=%.3f\n",
                                 k.max_n, t.layout, t.block_size, t.variant, ms);
                if (best < 0 || ms < best) {
                    best = ms;
                    best_lay = t.layout;
                    best_blk = t.block_size;
                    best_var = t.variant;
                }
            }
        }
        configure((int)c, best_lay, best_blk, best_var);
    }
    build_graph();
    tuned = true;
}

void Batch::apply_limits() {
    // classes that share a kernel need its largest shared-memory size and a carve-out that keeps
    // every class's resident blocks; kernel attributes are process-wide, so they are re-applied
    // before each launch of the graph
    // kernel numbers of sim_kernel_limits: 1 / 5 batched lane (plain / `_full`, variant: cooperative
    // update), 2 batched warp, 7 batched lane with global rows and 9 with global active words
    // (variant: `_full`)
    auto kernel_of = [](const Class& k) -> std::pair<int, int> {
        if (k.layout == MBG_LAYOUT_LANE && k.variant == 2) return {9, k.full ? 1 : 0};
        if (k.layout == MBG_LAYOUT_LANE) return {k.full ? 5 : 1, k.variant == 1 ? 1 : 0};
        if (k.layout == MBG_LAYOUT_LANE_GLOBAL) return {7, k.full ? 1 : 0};
        return {2, k.variant ? 1 : 0};
    };
    for (int kern : {1, 2, 5, 7, 9}) {
        for (int var = 0; var < 2; ++var) {
            std::vector<int> blocks, want;
            std::vector<size_t> smems;
            for (const Class& k : classes) {
                if (kernel_of(k) != std::make_pair(kern, var)) continue;
                blocks.push_back(k.block);
                smems.push_back(k.smem);
                want.push_back(std::max(1, k.grid / std::max(1, sms)));
            }
            if (!blocks.empty())
                ck(sim_kernel_limits(kern, var != 0, blocks.data(), smems.data(), want.data(), (int)blocks.size()),
                   "batched kernel attributes");
        }
    }
}

void Batch::run(cudaStream_t stream) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    cudaGetLastError();  // drop a stale non-sticky error of an earlier unrelated call
    std::unique_lock<std::mutex> lock(kernel_attr_mutex());
    if (opts.autotune && !tuned) autotune();
    cudaStream_t s = stream ? stream : capture_stream;
    apply_limits();
    ck(cudaEventRecord(ev0, s), "cudaEventRecord");
    ck(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
    lock.unlock();
    ck(cudaEventRecord(ev1, s), "cudaEventRecord");
    ck(cudaStreamSynchronize(s), "batched simulation");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
    double kms = 0;
    for (Class& k : classes) {
        ck(cudaEventElapsedTime(&k.kernel_ms, k.e0, k.e1), "cudaEventElapsedTime");
        kms += k.kernel_ms;
    }
    summary = mbg_run_summary{};
    uint32_t err = 0;
    int layouts = 0;
    for (Inst& x : inst) {
        const Class& k = classes[x.cls];
        const unsigned long long* c = reinterpret_cast<const unsigned long long*>(small_host + x.small_off);
        uint32_t flags[2];
        std::memcpy(flags, small_host + x.small_off + 8 * CNT_COUNT, 8);
        mbg_run_summary& r = x.summary;
        r = mbg_run_summary{};
        r.trajectories = x.n_traj;
        r.transitions = c[CNT_TRANSITIONS];
        r.steps = c[CNT_STEPS];
        r.finished = c[CNT_FINISHED];
        r.fixed_points = c[CNT_FIXED];
        r.step_limited = c[CNT_STEP_LIMIT];
        r.errors = c[CNT_ERROR];
        r.device_error = flags[0];
        r.fixed_point_states = flags[1];
        r.layout = k.layout;
        r.block_size = k.block;
        r.grid_size = k.grid;
        // as mbg_sim_opts::lane_update: 0 cooperative, 1 per-lane, 2 per-lane with global active words
        r.lane_update = k.layout == MBG_LAYOUT_LANE ? (k.variant == 2 ? 2 : k.variant == 1 ? 0 : 1)
                        : k.layout == MBG_LAYOUT_LANE_GLOBAL ? 1 : 0;
        r.kernel_ms = k.kernel_ms;
        summary.trajectories += r.trajectories;
        summary.transitions += r.transitions;
        summary.steps += r.steps;
        summary.finished += r.finished;
        summary.fixed_points += r.fixed_points;
        summary.step_limited += r.step_limited;
        summary.errors += r.errors;
        summary.fixed_point_states += r.fixed_point_states;
        err |= flags[0];
        layouts |= 1 << k.layout;
        x.fetched = false;
    }
    summary.device_error = err;
    // one layout for every class, or 0 when the classes differ
    summary.layout = (layouts & (layouts - 1)) ? 0 : __builtin_ctz((unsigned)layouts);
    summary.sim_ms = ms;
    summary.kernel_ms = kms;
    ran = true;
    if (err) throw DeviceError("device error flags 0x" + std::to_string(err));
}

void Batch::fetch(int i) {
    if (!ran) throw StateError("results requested before mbg_batch_run");
    if (i < 0 || i >= (int)inst.size()) throw ArgError("instance index out of range");
    Inst& x = inst[i];
    if (x.fetched) return;
    ck(cudaSetDevice(device), "cudaSetDevice");
    const uint64_t S = 1ull << x.cm.n_out;
    x.hist.resize(x.cm.windows * S);
    x.th.resize(x.cm.windows);
    x.fin.resize(S);
    ck(cudaMemcpy(x.hist.data(), x.prm.hist, x.hist.size() * 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    ck(cudaMemcpy(x.th.data(), x.prm.th_hist, x.th.size() * 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    ck(cudaMemcpy(x.fin.data(), x.prm.final_hist, x.fin.size() * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    const size_t nu = x.summary.fixed_point_states;
    x.fp_words.resize(nu * x.cm.words);
    x.fp_cnt.resize(nu);
    if (nu) {
        ck(cudaMemcpy(x.fp_words.data(), x.fp.out_states, x.fp_words.size() * 4, cudaMemcpyDeviceToHost),
           "cudaMemcpy D2H");
        ck(cudaMemcpy(x.fp_cnt.data(), x.fp.out_cnt, nu * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    }
    x.fetched = true;
}

void Batch::window_sums(int w, std::vector<uint64_t>& out) {
    if (!ran) throw StateError("results requested before mbg_batch_run");
    ck(cudaSetDevice(device), "cudaSetDevice");
    std::vector<WindowSpan> spans(inst.size());
    uint64_t total = 0, max_n = 0;
    for (size_t i = 0; i < inst.size(); ++i) {
        const Inst& x = inst[i];
        const int wi = w < 0 ? x.cm.windows + w : w;
        if (wi < 0 || wi >= x.cm.windows)
            throw ArgError("window " + std::to_string(w) + " out of range for instance " + std::to_string(i));
        const uint64_t S = 1ull << x.cm.n_out;
        spans[i] = WindowSpan{x.prm.hist + (size_t)wi * S, total, S};
        total += S;
        max_n = std::max(max_n, S);
    }
    out.resize(total);
    if (spans.empty()) return;
    struct Blocks {  // returned to the block cache however the gather ends (the copies are synchronous)
        void* spans = nullptr;
        void* sums = nullptr;
        ~Blocks() {
            dev_free(spans);
            dev_free(sums);
        }
    } b;
    b.spans = dev_alloc(spans.size() * sizeof(WindowSpan), "window spans");
    b.sums = dev_alloc(total * 8, "gathered window sums");
    ck(cudaMemcpy(b.spans, spans.data(), spans.size() * sizeof(WindowSpan), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ck(launch_window_gather(static_cast<const WindowSpan*>(b.spans), (int)spans.size(), max_n,
                            static_cast<unsigned long long*>(b.sums), nullptr),
       "window gather");
    ck(cudaMemcpy(out.data(), b.sums, total * 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
}

}  // namespace mbg
