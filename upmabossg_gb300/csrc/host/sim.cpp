// Simulation handle: device image of the model, result buffers, kernel choice and launch.
//
// Replaces the batch runner src/simulation_runner.cu:54-180 (segments of <= 99 steps, trajectory
// buffers, thrust partitions and refills between launches) with one persistent launch in which
// every warp (or thread) pulls trajectory ids from a work counter until none are left, plus the
// statistics objects of src/statistics/ whose work happens inside that launch.
#include "sim.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <tuple>

#include "../device/kernels.h"
#include "devmem.hpp"

namespace mbg {

namespace {

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
T* dalloc(size_t n, std::vector<void*>& owned) {
    void* p = dev_alloc((n ? n : 1) * sizeof(T), "simulation buffer");
    owned.push_back(p);
    return static_cast<T*>(p);
}

template <class T>
T* upload(const std::vector<T>& v, std::vector<void*>& owned) {
    T* p = dalloc<T>(v.size(), owned);
    if (!v.empty()) ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    return p;
}

}  // namespace

uint32_t fp_slot_count(uint64_t capacity) {
    if (capacity > kMaxTrajectories)
        throw ArgError("fixed-point capacity " + std::to_string(capacity) + " above the limit of 2^30 entries");
    uint64_t p = 1024;
    while (p < 2 * capacity) p <<= 1;
    return (uint32_t)p;  // <= 2^31
}

DeviceLayout layout_model(const CompiledModel& cm) {
    DeviceLayout d;
    d.nodes.resize(cm.n);
    d.tab_off.assign(cm.n, 0);
    d.pal_off.assign(cm.n, 0);
    for (int i = 0; i < cm.n; ++i) {
        const CompiledNode& cn = cm.nodes[i];
        DevNode& dn = d.nodes[i];
        std::memset(&dn, 0, sizeof dn);
        dn.reg_off = (uint32_t)d.regs.size();
        for (int r : cn.regs) d.regs.push_back((uint16_t)r);
        for (size_t j = 0; j < cn.regs.size() && j < (size_t)kInlineRegs; ++j) dn.r[j] = (uint16_t)cn.regs[j];
        dn.k = (uint16_t)cn.regs.size();
        dn.kind = (uint16_t)cn.kind;
        if (cn.kind == NODE_BINARY) {
            dn.tab_off = (uint32_t)d.tabs.size();
            d.tabs.insert(d.tabs.end(), cn.bits.begin(), cn.bits.end());
            dn.up = cn.up;
            dn.down = cn.down;
            if (cn.regs.size() <= 5) {
                dn.table = cn.bits[0];
                if (cn.bits.size() > 1) dn.table |= (uint64_t)cn.bits[1] << 32;
            }
        } else {
            dn.tab_off = (uint32_t)d.pidx.size();
            d.pidx.insert(d.pidx.end(), cn.pidx.begin(), cn.pidx.end());
            dn.pal_off = (uint32_t)d.palette.size();
            d.palette.insert(d.palette.end(), cn.palette.begin(), cn.palette.end());
        }
        d.tab_off[i] = dn.tab_off;
        d.pal_off[i] = dn.pal_off;
        LaneNode ln;
        std::memset(&ln, 0, sizeof ln);
        ln.up = dn.up;
        ln.down = dn.down;
        ln.k = dn.k;
        for (size_t j = 0; j < cn.regs.size() && j < 4; ++j) ln.r[j] = (uint16_t)cn.regs[j];
        if (cn.kind != NODE_BINARY) {
            ln.flags = kLanePalette;
        } else if (cn.regs.size() > 12) {
            ln.flags = kLaneFar;
        } else if (cn.regs.size() > 4) {
            LaneWide w;
            std::memset(&w, 0, sizeof w);
            for (size_t j = 4; j < cn.regs.size(); ++j) w.r[j - 4] = (uint16_t)cn.regs[j];
            if (cn.regs.size() <= 6)
                for (size_t q = 0; q < cn.bits.size() && q < 4; ++q) w.table[q] = cn.bits[q];
            else
                w.table[0] = dn.tab_off;
            ln.flags = kLaneWideTable;
            ln.table = (uint32_t)d.lwide.size();
            d.lwide.push_back(w);
        } else {
            ln.table = cn.bits[0];
        }
        d.lnodes.push_back(ln);
    }
    d.dep_off.push_back(0);
    for (int i = 0; i < cm.n; ++i) {
        for (int x : cm.deps[i]) {
            const auto& regs = cm.nodes[x].regs;
            uint32_t pos = 0xFF;
            for (size_t j = 0; j < regs.size(); ++j)
                if (regs[j] == i) pos = (uint32_t)j;
            const uint32_t out = cm.out_pos[x] >= 0 ? 1u : 0u;
            d.deps.push_back(((uint32_t)x << 16) | (out << 15) | ((uint32_t)regs.size() << 8) | pos);
        }
        d.dep_off.push_back((uint32_t)d.deps.size());
    }
    for (int o : cm.out_nodes) d.out_nodes.push_back((uint16_t)o);
    for (int i = 0; i < cm.n; ++i) d.out_pos.push_back((int16_t)cm.out_pos[i]);
    d.istate_thr = cm.istate_thr;
    return d;
}

void check_layout(const CompiledModel& cm, const DeviceLayout& d) {
    const uint32_t n = (uint32_t)cm.n;
    auto need = [](bool ok, const char* what, uint32_t i) {
        if (!ok) throw ModelError(std::string("device layout check: ") + what + " (node " + std::to_string(i) + ")");
    };
    need(d.nodes.size() == n && d.lnodes.size() == n && d.out_pos.size() == n && d.istate_thr.size() == n,
         "per-node arrays sized to the model", 0);
    need(d.dep_off.size() == n + 1 && d.dep_off[n] == d.deps.size(), "dependency offsets", n);
    for (uint32_t i = 0; i < n; ++i) {
        const DevNode& dn = d.nodes[i];
        const LaneNode& ln = d.lnodes[i];
        const uint32_t k = dn.k;
        need(k == cm.nodes[i].regs.size() && ln.k == k, "regulator count", i);
        need((uint64_t)dn.reg_off + k <= d.regs.size(), "regulator list inside regs", i);
        for (uint32_t j = 0; j < k; ++j) need(d.regs[dn.reg_off + j] < n, "regulator id", i);
        for (uint32_t j = 0; j < k && j < (uint32_t)kInlineRegs; ++j) need(dn.r[j] < n, "inline regulator id", i);
        for (uint32_t j = 0; j < k && j < 4; ++j) need(ln.r[j] < n, "lane-record regulator id", i);
        const uint64_t entries = 2ull << k;  // table assignments (self bit + k regulators)
        if (dn.kind == NODE_BINARY) {
            need((uint64_t)dn.tab_off + (entries + 31) / 32 <= d.tabs.size(), "truth table inside tabs", i);
            need(ln.flags == 0u || ln.flags == kLaneWideTable || ln.flags == kLaneFar, "lane-record kind", i);
            need((ln.flags == 0u) == (k <= 4), "lane-record inline table", i);
            if (ln.flags == kLaneWideTable) {
                need(k > 4 && k <= 12 && ln.table < d.lwide.size(), "side record index", i);
                const LaneWide& w = d.lwide[ln.table];
                for (uint32_t j = 4; j < k; ++j) need(w.r[j - 4] < n, "side-record regulator id", i);
                if (k > 6) need((uint64_t)w.table[0] + (entries + 31) / 32 <= d.tabs.size(), "side-record table", i);
            }
        } else {
            need(ln.flags == kLanePalette, "lane-record kind", i);
            need((uint64_t)dn.tab_off + entries <= d.pidx.size(), "palette indices inside pidx", i);
            const size_t np = cm.nodes[i].palette.size();
            need((uint64_t)dn.pal_off + np <= d.palette.size(), "palette inside palette array", i);
            for (uint64_t a = 0; a < entries; ++a) need(d.pidx[dn.tab_off + a] < np, "palette index", i);
        }
        need(d.dep_off[i] <= d.dep_off[i + 1], "dependency list order", i);
        for (uint32_t q = d.dep_off[i]; q < d.dep_off[i + 1]; ++q) {
            const uint32_t e = d.deps[q], dn_id = e >> 16, kd = (e >> 8) & 0x7fu, pos = e & 0xffu;
            need(dn_id < n, "dependency entry node", i);
            need(kd == d.nodes[dn_id].k, "dependency entry regulator count", i);
            need(pos == 0xffu ? dn_id == i : (pos < kd && d.regs[d.nodes[dn_id].reg_off + pos] == i),
                 "dependency entry position", i);
            need(((e >> 15) & 1u) == (cm.out_pos[dn_id] >= 0 ? 1u : 0u), "dependency entry output flag", i);
        }
    }
    need(d.out_nodes.size() == (size_t)cm.n_out, "output list", 0);
    for (size_t q = 0; q < d.out_nodes.size(); ++q) {
        need(d.out_nodes[q] < n && d.out_pos[d.out_nodes[q]] == (int16_t)q, "output node", (uint32_t)q);
    }
}

void set_model_constants(SimParams& prm, const CompiledModel& cm) {
    prm.n = cm.n;
    prm.words = cm.words;
    prm.n_out = cm.n_out;
    prm.windows = cm.windows;
    prm.frac_bits = cm.frac_bits;
    prm.discrete = cm.discrete ? 1 : 0;
    prm.max_time = cm.max_time;
    prm.tick = cm.tick;
    prm.has_palette = 0;
    for (auto& nd : cm.nodes) prm.has_palette |= nd.kind == NODE_PALETTE ? 1 : 0;
    // clock fraction bits: max_time + tick stays below 2^(61 - bits)
    const int tb = std::min(40, (int)std::floor(61.0 - std::log2(cm.max_time + cm.tick + 1.0)));
    if (tb < 32) throw ModelError("max_time too large for the fixed-point clock");
    prm.time_bits = tb;
    prm.max_time_fx = (unsigned long long)std::nearbyint(std::ldexp(cm.max_time, tb));
    prm.tick_fx = (unsigned long long)std::nearbyint(std::ldexp(cm.tick, tb));
    prm.to_real = std::ldexp(1.0f, -cm.frac_bits);
}

void check_model_limits(const CompiledModel& cm, uint64_t n_traj) {
    if (n_traj == 0) throw ArgError("no trajectories to simulate (n_traj and sample_count are 0)");
    if (n_traj > kMaxTrajectories) throw ArgError("more than 2^30 trajectories in one run");
    if (cm.n_out > 24) throw ModelError("more than 24 output nodes");
    const uint64_t hist_bytes = (uint64_t)cm.windows * (1ull << cm.n_out) * 8;
    if (hist_bytes > (16ull << 30)) throw ModelError("window histogram would exceed 16 GiB");
    if (!cm.discrete && (double)n_traj * cm.tick >= 2147483648.0)
        throw ModelError("n_traj x time_tick too large for the 2^-32 fixed-point window sums");
}

namespace {

void* raw_alloc(size_t bytes, const char* what) { return dev_alloc(bytes, what); }

// Returns a block to the cache once nothing can still be using it (a replacement in mid-life:
// the device is synchronised, as cudaFree would).
void free_now(void* p) {
    if (!p) return;
    cudaDeviceSynchronize();
    dev_free(p);
}

int ceil_log2_u64(uint64_t x) {
    int c = 0;
    while (c < 63 && (1ull << c) < x) ++c;
    return c;
}

// Window-table size learned by earlier runs of the process (auto mode), per model shape and
// trajectory-count class: log2 of the hash slots, or 0 for the dense table. A new handle of the
// same shape starts at the size that held, instead of growing (and re-running) again.
std::mutex g_window_mu;
std::map<std::tuple<int, int, int, int>, int> g_window_bits;

std::tuple<int, int, int, int> window_class(const CompiledModel& cm, uint64_t n_traj) {
    return {cm.n, cm.n_out, cm.windows, ceil_log2_u64(n_traj)};
}

constexpr uint64_t kDenseWindowMaxBytes = 2ull << 30;  // auto: dense tables up to 2 GiB
constexpr int kDefaultHashBits = 22;                    // 4 Mi slots, 64 MiB: fits in L2

}  // namespace

void Sim::choose_window_table() {
    n_bins = (uint64_t)cm.windows << cm.n_out;
    const int mode = opts.window_table;
    if (mode < 0 || mode > 2) throw ArgError("window_table must be 0 (auto), 1 (dense) or 2 (hash)");
    if (opts.window_hash_bits != 0 && (opts.window_hash_bits < 10 || opts.window_hash_bits > 31))
        throw ArgError("window_hash_bits must be 0 or within 10..31");
    const bool hash_ok = n_bins <= (1ull << 31);  // bins as u32 in the compacted read-back
    if (mode == 2 && !hash_ok) throw ModelError("window hash table: more than 2^31 (window, output state) bins");
    // Measured on the GB300 (20-node workload, 100 windows x 2^20 states, 839 MB dense): the dense
    // table's fire-and-forget atomics keep the simulation kernel at 0.9 ms, while the hash table's
    // claim-or-match waits on an L2 round trip per flush (1.5-1.9 ms); the read-back is compacted on
    // the device either way. So the dense table is used while it is affordable and the hash table
    // only beyond that, where it holds what a run reaches: every trajectory holds at least one
    // output state per window, so trajectories x windows estimates the reached bins.
    // the warp layout runs on the dense table only (its hash-table form could stall the GPU when the
    // table overflowed): a run that asks for it keeps the dense table at any size
    const bool warp = opts.layout == MBG_LAYOUT_WARP;
    if (warp && mode == 2)
        throw ArgError("the warp layout uses the dense window table only (window_table = 1 or 0, or another layout)");
    const uint64_t est = std::min<uint64_t>(n_bins, n_traj * (uint64_t)cm.windows);
    const bool hash = mode == 2 || (mode == 0 && !warp && hash_ok && n_bins * 8 > kDenseWindowMaxBytes);
    int bits = 0;
    if (hash) {
        bits = std::min(kDefaultHashBits, std::max(10, ceil_log2_u64(2 * est)));
        if (opts.window_hash_bits) {
            bits = opts.window_hash_bits;
        } else if (mode == 0) {
            std::lock_guard<std::mutex> lock(g_window_mu);
            auto it = g_window_bits.find(window_class(cm, n_traj));
            if (it != g_window_bits.end()) bits = it->second;
        }
    }
    if (bits == 0)
        set_window_table(0);
    else
        grow_window_table(bits);  // dense instead when the hash table would be the larger
}

void Sim::set_window_table(int bits) {
    if (hslots) {
        free_now(hslots);
        hslots = nullptr;
    }
    if (bits == 0) {
        if (!dense_hist)
            dense_hist = static_cast<unsigned long long*>(raw_alloc(n_bins * 8, "dense window table"));
    } else {
        if (dense_hist) {
            free_now(dense_hist);
            dense_hist = nullptr;
        }
        hslots = static_cast<unsigned long long*>(raw_alloc((size_t)16 << bits, "window hash table"));
    }
    hash_bits = bits;
    prm.hist = dense_hist;
    prm.hslots = hslots;
    prm.hash_bits = bits;
}

// A larger hash table for the next run: 2^bits slots, or (auto mode) the dense table once the
// hash table would take more than half of the dense table's bytes.
void Sim::grow_window_table(int bits) {
    const bool forced = opts.window_table == 2;
    if (!forced && (bits > 31 || ((uint64_t)16 << bits) > n_bins * 4)) {
        set_window_table(0);
        return;
    }
    if (bits > 31) throw ModelError("window hash table: more than 2^31 slots needed");
    set_window_table(bits);
}

Sim::~Sim() {
    // the blocks go back to the process cache: nothing may still use them (cudaFree synchronised
    // the device implicitly; the cache does not)
    if (!owned.empty()) cudaDeviceSynchronize();
    for (void* p : {(void*)dense_hist, (void*)hslots, (void*)wc_bitmap, (void*)wc_wpre, (void*)wc_chunk,
                    (void*)wc_total, (void*)wc_bin, (void*)wc_sum, (void*)fc_state, (void*)fc_count,
                    (void*)lane_state})
        dev_free(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (evk0) cudaEventDestroy(evk0);
    if (evk1) cudaEventDestroy(evk1);
    pinned_free(host_small);
    for (void* p : owned) dev_free(p);
}

void Sim::create(const CompiledModel& model, const std::vector<std::string>& node_names, const mbg_sim_opts& o) {
    cm = model;
    names = node_names;
    opts = o;
    n_traj = o.n_traj ? o.n_traj : cm.sample_count;
    seed = o.use_cfg_seed ? cm.seed : o.seed;
    check_model_limits(cm, n_traj);
    const uint64_t S = 1ull << cm.n_out;
    // option checks come before any device call
    if (o.block_size && (o.block_size % 32 != 0 || o.block_size > 256))
        throw ArgError("block_size must be a multiple of 32, at most 256");
    if (o.layout < MBG_LAYOUT_AUTO || o.layout > MBG_LAYOUT_LANE_GLOBAL) throw ArgError("unknown layout");
    if (o.lane_update < 0 || o.lane_update > 2) throw ArgError("lane_update must be 0, 1 or 2");
    if (o.layout == MBG_LAYOUT_THREAD && cm.words > 16) throw ModelError("thread layout supports at most 512 nodes");
    if (o.redraw_period && (o.layout == MBG_LAYOUT_LANE || o.layout == MBG_LAYOUT_LANE_GLOBAL))
        throw ArgError("redraw_period is supported by the thread and warp layouts");

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw CudaError("no CUDA device available");
    }
    device = o.device;
    if (device < 0 || device >= ndev) throw ArgError("device ordinal out of range");
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");

    dl = layout_model(cm);
    check_layout(cm, dl);
    // model arrays
    std::memset(&prm, 0, sizeof prm);
    prm.nodes = upload(dl.nodes, owned);
    prm.lnodes = upload(dl.lnodes, owned);
    prm.lwide = upload(dl.lwide, owned);
    prm.regs = upload(dl.regs, owned);
    prm.tabs = upload(dl.tabs, owned);
    prm.pidx = upload(dl.pidx, owned);
    prm.palette = reinterpret_cast<const unsigned long long*>(upload(dl.palette, owned));
    prm.dep_off = upload(dl.dep_off, owned);
    prm.deps = upload(dl.deps, owned);
    prm.out_nodes = upload(dl.out_nodes, owned);
    prm.out_pos = upload(dl.out_pos, owned);
    prm.istate_thr = upload(dl.istate_thr, owned);
    set_model_constants(prm, cm);
    lane_full = prm.has_palette || cm.max_k > 12;
    prm.max_steps = o.max_steps ? o.max_steps : 0xFFFFFFFFu;
    prm.redraw_period = o.redraw_period;
    prm.seed = seed;
    prm.n_traj = n_traj;
    prm.traj_base = o.traj_base;
    // results
    choose_window_table();
    prm.th_hist = dalloc<unsigned long long>((size_t)cm.windows, owned);
    prm.final_hist = dalloc<unsigned int>((size_t)S, owned);
    fp_capacity = (uint32_t)n_traj;
    prm.fp_capacity = fp_capacity;
    prm.fp_states = dalloc<unsigned int>((size_t)fp_capacity * cm.words, owned);
    prm.fp_count = dalloc<unsigned int>(1, owned);
    prm.counters = dalloc<unsigned long long>(CNT_COUNT, owned);
    prm.error_flag = dalloc<unsigned int>(1, owned);
    if (o.record_trajectories) {
        prm.traj_state = dalloc<unsigned int>((size_t)n_traj * cm.words, owned);
        prm.traj_time = dalloc<double>((size_t)n_traj, owned);
        prm.traj_transitions = dalloc<unsigned int>((size_t)n_traj, owned);
        prm.traj_status = dalloc<unsigned char>((size_t)n_traj, owned);
    }
    n_slots = fp_slot_count(fp_capacity);
    slot_rep = dalloc<unsigned int>(n_slots, owned);
    slot_cnt = dalloc<unsigned int>(n_slots, owned);
    fp_out_states = dalloc<unsigned int>((size_t)fp_capacity * cm.words, owned);
    fp_out_cnt = dalloc<unsigned int>(fp_capacity, owned);
    fp_unique = dalloc<unsigned int>(1, owned);
    host_small = pinned_alloc(256);
    ck(cudaEventCreate(&ev0), "cudaEventCreate");
    ck(cudaEventCreate(&ev1), "cudaEventCreate");
    ck(cudaEventCreate(&evk0), "cudaEventCreate");
    ck(cudaEventCreate(&evk1), "cudaEventCreate");

    if (o.layout != MBG_LAYOUT_AUTO) {
        int blk = o.block_size;
        if (blk <= 0) {
            // the lane layout's shared memory grows with N: the largest block that fits
            blk = 256;
            if (o.layout == MBG_LAYOUT_LANE)
                while (blk > 32 && (o.lane_update == 2 ? sim_lane_split_smem(cm.n, blk) : sim_lane_smem(cm.n, blk)) >
                                       227 * 1024)
                    blk >>= 1;
        }
        setup_layout(o.layout, blk, o.lane_update);
    } else if (o.thread_cutoff > 0) {
        const int big = hash_bits > 0 ? MBG_LAYOUT_LANE_GLOBAL : MBG_LAYOUT_WARP;  // warp: dense table only
        const int lay = cm.words <= 16 && cm.n <= o.thread_cutoff ? MBG_LAYOUT_THREAD : big;
        setup_layout(lay, o.block_size > 0 ? o.block_size : 256, 1);
    } else {
        autotune();
    }
}

namespace {
// Autotuned launch shapes per (model size class ceil(log2 N), class ceil(log2 n) of the longest
// pilot, redraw_period set, window hash table), shared by all simulations of the process: layout,
// threads per block and the lane layout's reader update.
std::mutex g_tune_mu;
struct Shape {
    int layout, block;
    int update;  // the lane layout's reader update (mbg_sim_opts::lane_update); 1 for the others
};
std::map<std::tuple<int, int, int, int>, Shape> g_tuned;

int ceil_log2(uint64_t x) {
    int c = 0;
    while ((1ull << c) < x) ++c;
    return c;
}

// Tuned shapes also persist on disk, one line per (GPU, library build, class), so that a new
// process (a command-line run, say) finds them without timing the pilots again. A line from
// another GPU model or another build of the library never matches.
std::string tune_key(int device, const std::tuple<int, int, int, int>& cls) {
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return std::string();
    std::string name = prop.name;
    for (char& c : name)
        if (c == '|') c = '_';
    std::string key = name + "|" + std::to_string(prop.multiProcessorCount) + "|" + __DATE__ + "_" + __TIME__ + "|" +
                      std::to_string(std::get<0>(cls)) + "|" + std::to_string(std::get<1>(cls)) + "|" +
                      std::to_string(std::get<2>(cls)) + "|" + std::to_string(std::get<3>(cls));
    // one whitespace-free token per line (the device name and __DATE__ hold spaces)
    for (char& c : key)
        if (std::isspace((unsigned char)c)) c = '_';
    return key;
}

std::string tune_path() { return cache_dir() + "/autotune_v2.txt"; }

bool tune_lookup_disk(const std::string& key, Shape& out) {
    if (key.empty() || std::getenv("MBG_AUTOTUNE_NOCACHE")) return false;
    std::ifstream f(tune_path());
    std::string k;
    int lay = 0, blk = 0, upd = 0;
    bool found = false;
    while (f >> k >> lay >> blk >> upd)  // the last line for a key wins
        if (k == key) {
            out = Shape{lay, blk, upd};
            found = true;
        }
    return found;
}

void tune_store_disk(const std::string& key, const Shape& s) {
    if (key.empty() || std::getenv("MBG_AUTOTUNE_NOCACHE")) return;
    cache_mkdirs(cache_dir());
    std::ofstream f(tune_path(), std::ios::app);
    f << key << " " << s.layout << " " << s.block << " " << s.update << "\n";
}
}  // namespace

void Sim::autotune() {
    // the pilot is large enough to fill the GPU in every layout (or the whole run when smaller),
    // so that the choice reflects occupancy as well as per-transition cost
    const uint64_t pilot = std::min<uint64_t>(n_traj, 1u << 17);
    // the closest candidates again on a longer pilot: the run itself, up to 2^20 trajectories
    const uint64_t pilot2 = std::min<uint64_t>(n_traj, 8 * pilot);
    // the lane layout has no redraw_period and the warp layout no window hash table: such runs are
    // tuned (and cached) apart
    const std::tuple<int, int, int, int> cls{ceil_log2((uint64_t)cm.n), ceil_log2(pilot2), opts.redraw_period ? 1 : 0,
                                             hash_bits > 0 ? 1 : 0};
    const std::string key = tune_key(device, cls);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(cls);
        Shape disk{};
        if (it == g_tuned.end() && tune_lookup_disk(key, disk)) it = g_tuned.emplace(cls, disk).first;
        if (it != g_tuned.end()) {
            setup_layout(it->second.layout, opts.block_size > 0 ? opts.block_size : it->second.block,
                         it->second.update);
            return;
        }
    }
    // time every layout and block size on the pilot; all give identical results, so the kernel
    // times compare the same work
    struct PilotScope {  // the pilot's trajectory count, restored however the timing ends
        SimParams& p;
        uint64_t saved;
        PilotScope(SimParams& q, uint64_t n) : p(q), saved(q.n_traj) { p.n_traj = n; }
        ~PilotScope() { p.n_traj = saved; }
    } scope(prm, pilot);
    const bool log = std::getenv("MBG_AUTOTUNE_LOG") != nullptr;
    double best = -1;
    Shape best_shape{MBG_LAYOUT_WARP, 256, 1};
    std::vector<std::pair<double, Shape>> timed;
    for (int lay : {MBG_LAYOUT_THREAD, MBG_LAYOUT_WARP, MBG_LAYOUT_LANE, MBG_LAYOUT_LANE_GLOBAL}) {
        for (int blk : {64, 128, 256}) {
            for (int upd = 0; upd < 3; ++upd) {
                if (opts.block_size > 0 && blk != opts.block_size) continue;
                if (lay != MBG_LAYOUT_LANE && (blk == 64 || upd != 1)) continue;
                if (lay == MBG_LAYOUT_LANE_GLOBAL && opts.redraw_period) continue;
                if (lay == MBG_LAYOUT_WARP && hash_bits > 0) continue;  // dense window table only
                if (lay == MBG_LAYOUT_THREAD && cm.words > 16) continue;
                if (lay == MBG_LAYOUT_LANE && opts.redraw_period) continue;
                // the lane layout's rows in shared memory; the active-word rows in global memory
                // (update 2) only in blocks of 128 and 256
                if (lay == MBG_LAYOUT_LANE && upd < 2 && sim_lane_smem(cm.n, blk) > 227 * 1024) continue;
                if (lay == MBG_LAYOUT_LANE && upd == 2 && (blk == 64 || sim_lane_split_smem(cm.n, blk) > 227 * 1024))
                    continue;
                try {
                    setup_layout(lay, blk, upd);
                } catch (const JitError&) {
                    continue;  // a thread-layout kernel NVRTC cannot build: the other layouts remain
                }
                run(nullptr);  // warm-up (and JIT load)
                run(nullptr);
                if (log)
                    std::fprintf(stderr, "mbg autotune: n=%d pilot=%llu layout=%d block=%d update=%d kernel_ms=%.3f\n",
                                 cm.n, (unsigned long long)pilot, lay, blk, upd, summary.kernel_ms);
                timed.push_back({summary.kernel_ms, Shape{lay, blk, upd}});
                if (best < 0 || summary.kernel_ms < best) {
                    best = summary.kernel_ms;
                    best_shape = Shape{lay, blk, upd};
                }
            }
        }
    }
    // A short pilot starts every lane's first trajectory together; a long run reaches a steady
    // state in which the lanes of a warp are at unrelated points of their trajectories, and the
    // layouts rank differently there (as do layouts that hold different numbers of trajectories
    // resident: on the 1000-node workload the active words in global memory hold 768 per SM
    // against 512, 20% slower on 2^17 trajectories, even on 2^19, 4% faster on 10^6). The closest
    // candidates are timed again on a pilot up to eight times longer.
    if (pilot2 > pilot && timed.size() > 1) {
        std::sort(timed.begin(), timed.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        scope.p.n_traj = pilot2;
        // the three fastest within 15%, and the fastest of every (layout, variant) within 30%: a
        // short pilot can misrank the reader-update variants
        std::vector<size_t> pick;
        for (size_t i = 0; i < timed.size(); ++i) {
            bool first_of_kind = true;
            for (size_t j = 0; j < i; ++j)
                if (timed[j].second.layout == timed[i].second.layout &&
                    timed[j].second.update == timed[i].second.update)
                    first_of_kind = false;
            if ((i < 3 && timed[i].first <= 1.15 * timed[0].first) ||
                (first_of_kind && timed[i].first <= 1.3 * timed[0].first))
                pick.push_back(i);
        }
        best = -1;
        for (size_t i : pick) {
            const Shape& sh = timed[i].second;
            setup_layout(sh.layout, sh.block, sh.update);
            run(nullptr);
            if (log)
                std::fprintf(stderr, "mbg autotune: n=%d pilot=%llu layout=%d block=%d update=%d kernel_ms=%.3f\n",
                             cm.n, (unsigned long long)pilot2, sh.layout, sh.block, sh.update, summary.kernel_ms);
            if (best < 0 || summary.kernel_ms < best) {
                best = summary.kernel_ms;
                best_shape = sh;
            }
        }
    }
    scope.p.n_traj = scope.saved;
    ran = false;
    setup_layout(best_shape.layout, best_shape.block, best_shape.update);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[cls] = best_shape;
    tune_store_disk(key, best_shape);
}

void Sim::setup_layout(int lay, int blk, int update) {
    layout = lay;
    block = blk;
    lane_coop = update == 0;
    lane_split = lay == MBG_LAYOUT_LANE && update == 2;
    int bps = 0;
    if (layout == MBG_LAYOUT_THREAD) {
        double ms = 0;
        thread_kernel = jit_thread_kernel(generate_thread_model(cm, dl), ms);
        jit_ms += ms;
        smem = 0;
        ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)thread_kernel, block, 0),
           "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    } else if (layout == MBG_LAYOUT_LANE_GLOBAL) {
        smem = 0;
        lane_coop = false;  // per-lane reader update only
        ck(sim_lane_global_configure(lane_full, block, &bps), "configuring mbg_sim_lane_global");
    } else if (layout == MBG_LAYOUT_LANE) {
        smem = lane_split ? sim_lane_split_smem(cm.n, block) : sim_lane_smem(cm.n, block);
        if (smem > 227 * 1024) throw ModelError("model too large for the lane layout's shared memory at this block size");
        if (lane_split)
            ck(sim_lane_split_configure(lane_full, smem, block, &bps), "configuring mbg_sim_lane_split");
        else
            ck(sim_lane_configure(lane_coop, lane_full, smem, block, &bps), "configuring mbg_sim_lane");
    } else {
        // keep every node's regulator index in shared memory while a block's share stays small
        // enough for several resident blocks per SM; otherwise re-gather it on each update
        cached_index = (size_t)(block / 32) * sim_warp_smem_per_warp(cm.n, true) <= 64 * 1024;
        smem = (size_t)(block / 32) * sim_warp_smem_per_warp(cm.n, cached_index);
        if (smem > 227 * 1024) throw ModelError("model too large for the warp layout's shared memory");
        ck(sim_warp_configure(cached_index, smem), "cudaFuncSetAttribute");
        ck(sim_warp_occupancy(cached_index, block, smem, &bps), "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
    if (bps < 1) throw CudaError("kernel cannot be resident with this block size");
    if (opts.blocks_per_sm > 0) bps = std::min(bps, (int)opts.blocks_per_sm);
    grid = sms * bps;
    if (layout == MBG_LAYOUT_LANE_GLOBAL || (layout == MBG_LAYOUT_LANE && lane_split)) {
        // every resident block's rows (all of them, or the active words), each block's share
        // 256-byte aligned
        const uint64_t rows = layout == MBG_LAYOUT_LANE ? (uint64_t)sim_lane_rows(cm.n) * 4 * block
                                                        : sim_lane_smem(cm.n, block);
        const uint64_t block_bytes = (rows + 255) & ~(uint64_t)255;
        const uint64_t need = block_bytes * (uint64_t)grid;
        if (need > lane_state_bytes) {
            free_now(lane_state);
            lane_state = nullptr;
            lane_state_bytes = 0;
            lane_state = static_cast<unsigned char*>(dev_alloc(need, "lane layout rows"));
            lane_state_bytes = need;
        }
        prm.lane_state = lane_state;
        prm.lane_block_bytes = block_bytes;
    }
}

std::mutex& kernel_attr_mutex() {
    static std::mutex m;
    return m;
}

void Sim::run(cudaStream_t stream) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    window_reruns = 0;
    if (pending_hash_bits > 0) {  // the growth the last run asked for (its results are read by now)
        grow_window_table(pending_hash_bits);
        pending_hash_bits = 0;
    }
    for (;;) {
        launch(stream);
        const uint32_t err = summary.device_error;
        // a full hash table: nothing else went wrong, so the same run is repeated on a table four
        // times larger (every trajectory depends only on its id: the repeat is exact)
        if (hash_bits > 0 && err == (uint32_t)DEV_ERR_WINDOW_TABLE) {
            grow_window_table(hash_bits + 2);
            ++window_reruns;
            continue;
        }
        break;
    }
    summary.window_reruns = window_reruns;
    if (summary.device_error) throw DeviceError("device error flags 0x" + std::to_string(summary.device_error));
    // keep the table at most half full: the next run starts on a larger one (this run's results
    // stay in the current table until then)
    if (hash_bits > 0 && 2 * summary.window_entries > (1ull << hash_bits))
        pending_hash_bits = std::max(hash_bits + 1, ceil_log2_u64(2 * summary.window_entries));
    // the table that held, for the next automatic choice of this model shape (not a dense table the
    // warp layout kept regardless)
    if (opts.window_table == 0 && opts.window_hash_bits == 0 && opts.layout != MBG_LAYOUT_WARP) {
        std::lock_guard<std::mutex> lock(g_window_mu);
        g_window_bits[window_class(cm, n_traj)] = pending_hash_bits > 0 ? pending_hash_bits : hash_bits;
    }
}

void Sim::launch(cudaStream_t stream) {
    const uint64_t S = 1ull << cm.n_out;
    ck(cudaEventRecord(ev0, stream), "cudaEventRecord");
    if (hash_bits > 0)
        ck(cudaMemsetAsync(hslots, 0, (size_t)16 << hash_bits, stream), "cudaMemsetAsync");
    else
        ck(cudaMemsetAsync(dense_hist, 0, n_bins * 8, stream), "cudaMemsetAsync");
    ck(cudaMemsetAsync(prm.th_hist, 0, cm.windows * 8, stream), "cudaMemsetAsync");
    ck(cudaMemsetAsync(prm.final_hist, 0, S * 4, stream), "cudaMemsetAsync");
    ck(cudaMemsetAsync(prm.fp_count, 0, 4, stream), "cudaMemsetAsync");
    ck(cudaMemsetAsync(prm.counters, 0, CNT_COUNT * 8, stream), "cudaMemsetAsync");
    ck(cudaMemsetAsync(prm.error_flag, 0, 4, stream), "cudaMemsetAsync");
    ck(cudaEventRecord(evk0, stream), "cudaEventRecord");
    if (layout == MBG_LAYOUT_THREAD) {
        if (hash_bits > 0 && !thread_kernel_hash) {
            double ms = 0;
            thread_kernel_hash = jit_thread_kernel(generate_thread_model(cm, dl), ms, true);
            jit_ms += ms;
        }
        void* args[] = {(void*)&prm};
        ck(cudaLaunchKernel((const void*)(hash_bits > 0 ? thread_kernel_hash : thread_kernel), dim3(grid), dim3(block),
                            args, 0, stream),
           "cudaLaunchKernel(mbg_sim_thread)");
    } else {
        // kernel attributes are process-wide: re-apply this handle's before its launch
        std::lock_guard<std::mutex> lock(kernel_attr_mutex());
        const int want = std::max(1, grid / std::max(1, sms));
        if (layout == MBG_LAYOUT_LANE_GLOBAL) {
            ck(sim_kernel_limits(6, lane_full, &block, &smem, &want, 1, hash_bits > 0), "mbg_sim_lane_global attributes");
            ck(launch_sim_lane_global(prm, lane_full, grid, block, stream), "launch mbg_sim_lane_global");
        } else if (layout == MBG_LAYOUT_LANE && lane_split) {
            ck(sim_kernel_limits(8, lane_full, &block, &smem, &want, 1, hash_bits > 0), "mbg_sim_lane_split attributes");
            ck(launch_sim_lane_split(prm, lane_full, grid, block, smem, stream), "launch mbg_sim_lane_split");
        } else if (layout == MBG_LAYOUT_LANE) {
            ck(sim_kernel_limits(lane_full ? 4 : 0, lane_coop, &block, &smem, &want, 1, hash_bits > 0),
               "mbg_sim_lane attributes");
            ck(launch_sim_lane(prm, lane_coop, lane_full, grid, block, smem, stream), "launch mbg_sim_lane");
        } else {
            ck(sim_kernel_limits(3, cached_index, &block, &smem, &want, 1, hash_bits > 0), "mbg_sim_warp attributes");
            ck(launch_sim_warp(prm, cached_index, grid, block, smem, stream), "launch mbg_sim_warp");
        }
    }
    ck(cudaEventRecord(evk1, stream), "cudaEventRecord");
    ck(launch_fp_aggregate(prm.fp_states, prm.fp_count, fp_capacity, cm.words, slot_rep, slot_cnt, n_slots,
                           fp_out_states, fp_out_cnt, fp_unique, prm.error_flag, sms, stream),
       "launch fixed-point aggregation");
    ck(cudaEventRecord(ev1, stream), "cudaEventRecord");
    unsigned long long* hc = reinterpret_cast<unsigned long long*>(host_small);
    ck(cudaMemcpyAsync(hc, prm.counters, CNT_COUNT * 8, cudaMemcpyDeviceToHost, stream), "cudaMemcpyAsync");
    ck(cudaMemcpyAsync(hc + CNT_COUNT, prm.error_flag, 4, cudaMemcpyDeviceToHost, stream), "cudaMemcpyAsync");
    ck(cudaMemcpyAsync(reinterpret_cast<char*>(hc + CNT_COUNT) + 4, fp_unique, 4, cudaMemcpyDeviceToHost, stream),
       "cudaMemcpyAsync");
    ck(cudaStreamSynchronize(stream), "simulation kernel");
    float ms = 0, kms = 0;
    ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
    ck(cudaEventElapsedTime(&kms, evk0, evk1), "cudaEventElapsedTime");
    summary = mbg_run_summary{};
    summary.trajectories = n_traj;
    summary.transitions = hc[CNT_TRANSITIONS];
    summary.steps = hc[CNT_STEPS];
    summary.finished = hc[CNT_FINISHED];
    summary.fixed_points = hc[CNT_FIXED];
    summary.step_limited = hc[CNT_STEP_LIMIT];
    summary.errors = hc[CNT_ERROR];
    uint32_t flags[2];
    std::memcpy(flags, hc + CNT_COUNT, 8);
    summary.device_error = flags[0];
    summary.fixed_point_states = flags[1];
    summary.layout = layout;
    summary.sim_ms = ms;
    summary.kernel_ms = kms;
    summary.jit_ms = jit_ms;
    summary.block_size = block;
    summary.grid_size = grid;
    summary.lane_update = layout == MBG_LAYOUT_LANE ? (lane_split ? 2 : lane_coop ? 0 : 1)
                          : layout == MBG_LAYOUT_LANE_GLOBAL ? 1 : 0;
    summary.window_table = hash_bits > 0 ? 2 : 1;
    summary.window_hash_bits = hash_bits;
    summary.window_entries = hash_bits > 0 ? hc[CNT_WIN_ENTRIES] : 0;
    ran = true;
    fetched = false;
}

void Sim::compaction_scratch() {
    if (wc_bitmap) return;
    const uint64_t words = window_bitmap_words(n_bins);
    wc_bitmap = static_cast<unsigned*>(raw_alloc(words * 4, "window bitmap"));
    wc_wpre = static_cast<unsigned*>(raw_alloc(words * 4, "window bitmap prefixes"));
    wc_chunk = static_cast<unsigned*>(raw_alloc((size_t)window_chunks(n_bins) * 4, "window chunk prefixes"));
    wc_total = static_cast<unsigned long long*>(raw_alloc(8, "window bin count"));
}

void Sim::fetch() {
    if (!ran) throw StateError("results requested before mbg_sim_run");
    if (fetched) return;
    // MBG_FETCH_LOG=1: the host time of each read-back phase on stderr
    static const bool log = std::getenv("MBG_FETCH_LOG") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* what) {
        if (!log) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "mbg fetch: %s %.3f ms\n", what,
                     std::chrono::duration<double, std::milli>(now - t_last).count());
        t_last = now;
    };
    ck(cudaSetDevice(device), "cudaSetDevice");
    const uint64_t S = 1ull << cm.n_out;
    th.resize(cm.windows);
    ck(cudaMemcpy(th.data(), prm.th_hist, th.size() * 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    phase("transition entropy");
    // final states: the reached output states only
    fin_state.clear();
    fin_count.clear();
    if (S <= (1ull << 16)) {
        // at most 256 KiB of counts: read whole and compacted here
        std::vector<uint32_t> f(S);
        ck(cudaMemcpy(f.data(), prm.final_hist, S * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        for (uint64_t x = 0; x < S; ++x)
            if (f[x]) {
                fin_state.push_back((uint32_t)x);
                fin_count.push_back(f[x]);
            }
    } else {
        compaction_scratch();
        ck(launch_final_count(prm.final_hist, S, wc_bitmap, wc_wpre, wc_chunk, wc_total, sms, nullptr),
           "final-state compaction (count)");
        unsigned long long total = 0;
        ck(cudaMemcpy(&total, wc_total, 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        if (total > fc_cap) {
            free_now(fc_state);
            free_now(fc_count);
            fc_state = fc_count = nullptr;
            fc_cap = 0;
            fc_state = static_cast<unsigned*>(raw_alloc(total * 4, "compacted final states"));
            fc_count = static_cast<unsigned*>(raw_alloc(total * 4, "compacted final-state counts"));
            fc_cap = total;
        }
        if (total) {
            ck(launch_final_emit(prm.final_hist, S, wc_bitmap, wc_wpre, wc_chunk, fc_state, fc_count, sms, nullptr),
               "final-state compaction (emit)");
            fin_state.resize(total);
            fin_count.resize(total);
            ck(cudaMemcpy(fin_state.data(), fc_state, total * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
            ck(cudaMemcpy(fin_count.data(), fc_count, total * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        }
    }
    phase("final states");
    // window sums: the non-zero bins in increasing order
    wbin.clear();
    wsum.clear();
    if (hash_bits == 0 && n_bins <= (1ull << 20)) {
        // a small dense table (at most 8 MiB) is read whole and compacted here
        std::vector<uint64_t> h(n_bins);
        ck(cudaMemcpy(h.data(), dense_hist, n_bins * 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        for (uint64_t i = 0; i < n_bins; ++i)
            if (h[i]) {
                wbin.push_back((uint32_t)i);
                wsum.push_back(h[i]);
            }
    } else {
        // compacted on the device: only the reached bins are copied
        compaction_scratch();
        ck(launch_window_count(dense_hist, hslots, hash_bits, n_bins, wc_bitmap, wc_wpre, wc_chunk, wc_total, sms,
                               nullptr),
           "window compaction (count)");
        unsigned long long total = 0;
        ck(cudaMemcpy(&total, wc_total, 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        phase("window compaction: count");
        if (total > wc_cap) {
            free_now(wc_bin);
            free_now(wc_sum);
            wc_bin = nullptr;
            wc_sum = nullptr;
            wc_cap = 0;
            wc_bin = static_cast<unsigned*>(raw_alloc(total * 4, "compacted window bins"));
            wc_sum = static_cast<unsigned long long*>(raw_alloc(total * 8, "compacted window sums"));
            wc_cap = total;
        }
        if (total) {
            ck(launch_window_emit(dense_hist, hslots, hash_bits, n_bins, wc_bitmap, wc_wpre, wc_chunk, wc_bin, wc_sum,
                                  sms, nullptr),
               "window compaction (emit)");
            wbin.resize(total);
            wsum.resize(total);
            ck(cudaMemcpy(wbin.data(), wc_bin, total * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
            ck(cudaMemcpy(wsum.data(), wc_sum, total * 8, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        }
    }
    phase("window bins and sums");
    // first entry of every window: the bins are in increasing order, window w starts at w * 2^n_out
    wstart.assign((size_t)cm.windows + 1, 0);
    for (int w = 1; w <= cm.windows; ++w)
        wstart[w] = (size_t)(std::lower_bound(wbin.begin(), wbin.end(), (uint64_t)w << cm.n_out,
                                              [](uint32_t b, uint64_t v) { return (uint64_t)b < v; }) -
                             wbin.begin());
    phase("window index");
    // fixed points: representatives, counts, then their states
    const uint32_t nu = (uint32_t)summary.fixed_point_states;
    std::vector<uint32_t> words((size_t)nu * cm.words), cnt(nu);
    if (nu) {
        ck(cudaMemcpy(words.data(), fp_out_states, words.size() * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        ck(cudaMemcpy(cnt.data(), fp_out_cnt, nu * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    }
    fixed.clear();
    fixed.reserve(nu);
    for (uint32_t u = 0; u < nu; ++u) {
        FixedPoint f;
        f.words.assign(words.begin() + (size_t)u * cm.words, words.begin() + (size_t)(u + 1) * cm.words);
        f.count = cnt[u];
        fixed.push_back(std::move(f));
    }
    // order of static_state_t::operator< (state.h:38-45): highest word first
    std::sort(fixed.begin(), fixed.end(), [](const FixedPoint& a, const FixedPoint& b) {
        for (size_t w = a.words.size(); w-- > 0;)
            if (a.words[w] != b.words[w]) return a.words[w] < b.words[w];
        return false;
    });
    phase("fixed points");
    fetched = true;
}

}  // namespace mbg
