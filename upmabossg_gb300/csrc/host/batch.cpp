// Batched parameter sweeps: every instance's model image and results live in a few arenas, all
// instances run in one persistent launch of the warp-per-trajectory kernel, and the clearing,
// simulation, fixed-point aggregation and counter read-back are captured once into a CUDA graph.
// The reference has no batching: a sweep is one CLI run per instance (src/main.cpp:101-169),
// each with its own NVRTC compilation (src/kernel_compiler.cpp:61-164) and batch loop
// (src/simulation_runner.cu:54-180).
#include "batch.hpp"

#include <algorithm>
#include <cstring>

#include "../device/kernels.h"

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

uint32_t next_pow2(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return (uint32_t)p;
}

void* dmalloc(size_t bytes, std::vector<void*>& owned) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw NoMemError("cudaMalloc of " + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
    }
    owned.push_back(p);
    return p;
}

constexpr size_t kSmallPerInst = 96;  // 8 u64 counters, error word, unique fixed points

}  // namespace

Batch::~Batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    for (cudaEvent_t e : {ev0, ev1, evk0, evk1})
        if (e) cudaEventDestroy(e);
    if (small_host) cudaFreeHost(small_host);
    for (void* p : owned) cudaFree(p);
}

void Batch::create(const std::vector<const CompiledModel*>& models, const std::vector<uint64_t>& n_traj,
                   const std::vector<uint64_t>& seeds, const mbg_batch_opts& o) {
    if (models.empty()) throw ArgError("empty batch");
    opts = o;
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
    std::vector<DeviceLayout> dls(n);
    Layout ml, rl, pl, fl;
    struct Off {
        size_t nodes, lnodes, regs, tabs, pidx, palette, dep_off, deps, out_nodes, out_pos, istate;
        size_t hist, th, fin, fp_count, slot_cnt, rep, fp_states, out_states, out_cnt;
    };
    std::vector<Off> off(n);
    std::vector<unsigned long long> prefix(n + 1, 0);
    for (size_t i = 0; i < n; ++i) {
        Inst& x = inst[i];
        x.cm = *models[i];
        const CompiledModel& cm = x.cm;
        x.n_traj = n_traj.empty() || n_traj[i] == 0 ? cm.sample_count : n_traj[i];
        x.seed = seeds.empty() ? cm.seed : seeds[i];
        check_model_limits(cm, x.n_traj);
        if (cm.n_out > 32) throw ModelError("batched instances support at most 32 outputs");
        max_n = std::max(max_n, cm.n);
        prefix[i + 1] = prefix[i] + x.n_traj;
        dls[i] = layout_model(cm);
        const DeviceLayout& d = dls[i];
        Off& f = off[i];
        f.nodes = ml.add(d.nodes.size() * sizeof(DevNode));
        f.lnodes = ml.add(d.lnodes.size() * sizeof(LaneNode));
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
        x.fp.n_slots = std::max<uint32_t>(1024, next_pow2(2ull * cap));
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
    total_traj = prefix[n];
    small_bytes = n * kSmallPerInst + 8;  // + the work counter
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
    ck(cudaMallocHost((void**)&small_host, small_bytes), "cudaMallocHost");

    std::vector<SimParams> prms(n);
    std::vector<FpSlots> fps(n);
    for (size_t i = 0; i < n; ++i) {
        Inst& x = inst[i];
        const Off& f = off[i];
        SimParams& p = x.prm;
        std::memset(&p, 0, sizeof p);
        p.nodes = reinterpret_cast<const DevNode*>(model_arena + f.nodes);
        p.lnodes = reinterpret_cast<const LaneNode*>(model_arena + f.lnodes);
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
        prms[i] = p;
        fps[i] = x.fp;
    }
    d_params = static_cast<SimParams*>(dmalloc(n * sizeof(SimParams), owned));
    d_fps = static_cast<FpSlots*>(dmalloc(n * sizeof(FpSlots), owned));
    d_prefix = static_cast<unsigned long long*>(dmalloc((n + 1) * 8, owned));
    ck(cudaMemcpy(d_params, prms.data(), n * sizeof(SimParams), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ck(cudaMemcpy(d_fps, fps.data(), n * sizeof(FpSlots), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ck(cudaMemcpy(d_prefix, prefix.data(), (n + 1) * 8, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    desc.params = d_params;
    desc.prefix = d_prefix;
    desc.n_inst = (int)n;
    desc.work = reinterpret_cast<unsigned long long*>(small_dev + n * kSmallPerInst);

    ck(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (cudaEvent_t* e : {&ev0, &ev1, &evk0, &evk1}) ck(cudaEventCreate(e), "cudaEventCreate");
    const int blk = o.block_size > 0 ? o.block_size : 128;
    if (blk % 32 != 0 || blk > 256) throw ArgError("block_size must be a multiple of 32, at most 256");
    configure(blk, (size_t)(blk / 32) * sim_warp_batch_slice_bytes(max_n, true) <= 100 * 1024, o.blocks_per_sm);
}

void Batch::configure(int blk, bool cached, int blocks_per_sm) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    slice_bytes = sim_warp_batch_slice_bytes(max_n, cached);
    const size_t sm = (size_t)(blk / 32) * slice_bytes;
    if (sm > 227 * 1024) throw ModelError("largest instance too large for the batched warp layout");
    int bps = 0;
    ck(sim_warp_batch_configure(cached, sm, blk, &bps), "batched kernel occupancy");
    if (bps < 1) throw CudaError("batched kernel cannot be resident with this block size");
    if (blocks_per_sm > 0) bps = std::min(bps, blocks_per_sm);
    block = blk;
    cached_index = cached;
    smem = sm;
    grid = sms * bps;
    desc.slice_bytes = slice_bytes;
    build_graph();
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
    ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t e = cudaMemsetAsync(result_arena, 0, result_bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(rep_arena, 0xFF, rep_bytes, s);
    // external event-record nodes, so the kernel's own time can be read after each replay
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(evk0, s, cudaEventRecordExternal);
    if (e == cudaSuccess) e = launch_sim_warp_batch(desc, cached_index, grid, block, smem, s);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(evk1, s, cudaEventRecordExternal);
    if (e == cudaSuccess) e = launch_fp_aggregate_batch(d_params, d_fps, (int)inst.size(), 8, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(small_host, small_dev, small_bytes, cudaMemcpyDeviceToHost, s);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    ck(e, "capturing the batch graph");
    ck(e2, "cudaStreamEndCapture");
    graph = g;
    ck(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
}

void Batch::run(cudaStream_t stream) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    cudaGetLastError();  // drop a stale non-sticky error of an earlier unrelated call
    if (opts.autotune && !ran) autotune();
    cudaStream_t s = stream ? stream : capture_stream;
    ck(cudaEventRecord(ev0, s), "cudaEventRecord");
    ck(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
    ck(cudaEventRecord(ev1, s), "cudaEventRecord");
    ck(cudaStreamSynchronize(s), "batched simulation");
    float ms = 0, kms = 0;
    ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
    ck(cudaEventElapsedTime(&kms, evk0, evk1), "cudaEventElapsedTime");
    summary = mbg_run_summary{};
    uint32_t err = 0;
    for (Inst& x : inst) {
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
        r.layout = MBG_LAYOUT_WARP;
        summary.trajectories += r.trajectories;
        summary.transitions += r.transitions;
        summary.steps += r.steps;
        summary.finished += r.finished;
        summary.fixed_points += r.fixed_points;
        summary.step_limited += r.step_limited;
        summary.errors += r.errors;
        summary.fixed_point_states += r.fixed_point_states;
        err |= flags[0];
        x.fetched = false;
    }
    summary.device_error = err;
    summary.layout = MBG_LAYOUT_WARP;
    summary.sim_ms = ms;
    summary.kernel_ms = kms;
    ran = true;
    if (err) throw DeviceError("device error flags 0x" + std::to_string(err));
}

void Batch::autotune() {
    // Warps per block (= trajectories resident per block) and the shared-memory index cache,
    // timed on the full batch; the fastest shape is kept.
    const int blocks[3] = {64, 128, 256};
    double best = 1e30;
    int best_b = block;
    bool best_c = cached_index;
    for (int bi = 0; bi < 3; ++bi) {
        for (int c = 0; c < 2; ++c) {
            const bool cached = c == 1;
            tune_ms[bi][c] = -1;
            if ((size_t)(blocks[bi] / 32) * sim_warp_batch_slice_bytes(max_n, cached) > 100 * 1024) continue;
            configure(blocks[bi], cached, opts.blocks_per_sm);
            ck(cudaGraphLaunch(exec, capture_stream), "cudaGraphLaunch");
            ck(cudaEventRecord(ev0, capture_stream), "cudaEventRecord");
            ck(cudaGraphLaunch(exec, capture_stream), "cudaGraphLaunch");
            ck(cudaEventRecord(ev1, capture_stream), "cudaEventRecord");
            ck(cudaStreamSynchronize(capture_stream), "autotune run");
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
            tune_ms[bi][c] = ms;
            if (ms < best) {
                best = ms;
                best_b = blocks[bi];
                best_c = cached;
            }
        }
    }
    configure(best_b, best_c, opts.blocks_per_sm);
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

}  // namespace mbg
