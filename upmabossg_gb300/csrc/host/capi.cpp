// extern "C" surface of libmbg (declared in include/mbg.h). Every entry point catches, maps the
// error to an mbg_status and keeps the message for mbg_last_error(); nothing exits. The
// reference instead prints and calls exit() on any CUDA, NVRTC or parse error
// (src/utils.cpp:3-30, src/kernel_compiler.cpp:10-31, src/parser/driver.cpp:54-60).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <set>

#include "batch.hpp"
#include "sim.hpp"
#include "surrogate.hpp"

struct mbg_model {
    mbg::Model model;
    mbg::CompiledModel cm;
    std::vector<std::string> names;
};

struct mbg_sim {
    mbg::Sim sim;
};

struct mbg_batch {
    mbg::Batch batch;
};

struct mbg_surrogate {
    mbg::Surrogate s;
};

namespace {

thread_local std::string g_err;

mbg_status fail(mbg_status st, const std::string& msg) {
    g_err = msg;
    return st;
}

template <class F>
mbg_status guard(F&& f) {
    try {
        f();
        g_err.clear();
        return MBG_OK;
    } catch (const mbg::ArgError& e) {
        return fail(MBG_ERR_ARG, e.what());
    } catch (const mbg::IoError& e) {
        return fail(MBG_ERR_IO, e.what());
    } catch (const mbg::ModelError& e) {
        return fail(MBG_ERR_MODEL, e.what());
    } catch (const mbg::NoMemError& e) {
        return fail(MBG_ERR_NOMEM, e.what());
    } catch (const mbg::DeviceError& e) {
        return fail(MBG_ERR_DEVICE, e.what());
    } catch (const mbg::StateError& e) {
        return fail(MBG_ERR_STATE, e.what());
    } catch (const mbg::CudaError& e) {
        return fail(MBG_ERR_CUDA, e.what());
    } catch (const mbg::JitError& e) {
        return fail(MBG_ERR_JIT, e.what());
    } catch (const mbg::Error& e) {
        return fail(MBG_ERR_PARSE, e.what());
    } catch (const std::bad_alloc&) {
        return fail(MBG_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(MBG_ERR_ARG, e.what());
    }
}

mbg_status build_model(const std::string& bnd, const std::string& cfg, const std::string& bnd_name,
                       const std::string& cfg_name, mbg_model** out, const char* overrides = nullptr) {
    if (!out) return fail(MBG_ERR_ARG, "null output pointer");
    *out = nullptr;
    std::unique_ptr<mbg_model> m(new mbg_model());
    mbg_status st = guard([&] {
        mbg::parse_bnd(m->model, bnd, bnd_name);
        mbg::parse_cfg(m->model, cfg, cfg_name);
        if (overrides && *overrides) mbg::parse_cfg(m->model, overrides, "<overrides>");
    });
    if (st != MBG_OK) return st;
    st = guard([&] {
        try {
            m->cm = mbg::compile_model(m->model);
        } catch (const mbg::Error& e) {
            throw mbg::ModelError(e.what());
        }
        for (auto& n : m->model.nodes) m->names.push_back(n.name);
    });
    if (st != MBG_OK) return st;
    *out = m.release();
    return MBG_OK;
}

}  // namespace

namespace mbg {
mbg_status set_error(mbg_status st, const std::string& msg) { return fail(st, msg); }
}  // namespace mbg

extern "C" {

const char* mbg_last_error(void) { return g_err.c_str(); }

const char* mbg_version(void) { return "mbg-gb300 0.1 (sm_103a)"; }

int mbg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

mbg_status mbg_model_parse_files(const char* bnd_path, const char* cfg_path, mbg_model** out) {
    return mbg_model_parse_files_overrides(bnd_path, cfg_path, nullptr, out);
}

mbg_status mbg_model_parse_files_overrides(const char* bnd_path, const char* cfg_path, const char* cfg_overrides,
                                           mbg_model** out) {
    if (!bnd_path || !cfg_path) return fail(MBG_ERR_ARG, "null path");
    std::string bnd, cfg;
    try {
        bnd = mbg::read_file(bnd_path);
        cfg = mbg::read_file(cfg_path);
    } catch (const std::exception& e) {
        return fail(MBG_ERR_IO, e.what());
    }
    return build_model(bnd, cfg, bnd_path, cfg_path, out, cfg_overrides);
}

mbg_status mbg_model_parse_strings(const char* bnd_text, const char* cfg_text, mbg_model** out) {
    if (!bnd_text || !cfg_text) return fail(MBG_ERR_ARG, "null text");
    return build_model(bnd_text, cfg_text, "<bnd>", "<cfg>", out);
}

void mbg_model_destroy(mbg_model* m) { delete m; }

mbg_status mbg_model_from_arrays(int32_t n, const char* const* names, const int32_t* reg_off, const int32_t* regs,
                                 const uint32_t* logic, int64_t logic_words, const int64_t* logic_off,
                                 const double* rate_up, const double* rate_down, const double* istate,
                                 const uint8_t* is_output, const mbg_model_run* run, mbg_model** out) {
    if (!out) return fail(MBG_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!run) return fail(MBG_ERR_ARG, "null run constants");
    if (n < 1) return fail(MBG_ERR_ARG, "model has no nodes");
    std::unique_ptr<mbg_model> m(new mbg_model());
    mbg_status st = guard([&] {
        std::set<std::string> seen;
        for (int32_t i = 0; i < n; ++i) {
            std::string name = names ? (names[i] ? names[i] : "") : "N" + std::to_string(i);
            if (name.empty() || !seen.insert(name).second)
                throw mbg::ArgError("node names must be distinct and non-empty (node " + std::to_string(i) + ")");
            m->names.push_back(std::move(name));
        }
    });
    if (st != MBG_OK) return st;
    st = guard([&] {
        mbg::RunConstants rc;
        rc.max_time = run->max_time;
        rc.tick = run->time_tick;
        rc.sample_count = run->sample_count;
        rc.seed = run->seed;
        rc.discrete = run->discrete_time != 0;
        try {
            m->cm = mbg::compile_arrays(n, reg_off, regs, logic, logic_words, logic_off, rate_up, rate_down, istate,
                                        is_output, rc);
        } catch (const mbg::Error& e) {
            throw mbg::ModelError(e.what());
        }
    });
    if (st != MBG_OK) return st;
    *out = m.release();
    return MBG_OK;
}

mbg_status mbg_model_info_get(const mbg_model* m, mbg_model_info* out) {
    if (!m || !out) return fail(MBG_ERR_ARG, "null argument");
    const mbg::CompiledModel& cm = m->cm;
    std::memset(out, 0, sizeof *out);
    out->nodes = cm.n;
    out->words = cm.words;
    out->outputs = cm.n_out;
    out->windows = cm.windows;
    out->discrete_time = cm.discrete ? 1 : 0;
    out->frac_bits = cm.frac_bits;
    out->max_regulators = cm.max_k;
    for (auto& n : cm.nodes) out->palette_nodes += n.kind == mbg::NODE_PALETTE;
    out->max_time = cm.max_time;
    out->time_tick = cm.tick;
    out->sample_count = cm.sample_count;
    out->seed = cm.seed;
    return MBG_OK;
}

const char* mbg_model_node_name(const mbg_model* m, int32_t i) {
    if (!m || i < 0 || i >= (int32_t)m->names.size()) return nullptr;
    return m->names[i].c_str();
}

int32_t mbg_model_outputs(const mbg_model* m, int32_t* idx, int32_t cap) {
    if (!m) return -1;
    int32_t n = (int32_t)m->cm.out_nodes.size();
    for (int32_t i = 0; i < n && i < cap && idx; ++i) idx[i] = m->cm.out_nodes[i];
    return n;
}

mbg_status mbg_model_rate(const mbg_model* m, int32_t node, const uint8_t* state, uint64_t* fixed_rate,
                          double* rate) {
    if (!m || !state) return fail(MBG_ERR_ARG, "null argument");
    const mbg::CompiledModel& cm = m->cm;
    if (node < 0 || node >= cm.n) return fail(MBG_ERR_ARG, "node index out of range");
    const mbg::CompiledNode& cn = cm.nodes[node];
    const int k = (int)cn.regs.size();
    uint64_t a = state[node] ? (1ull << k) : 0ull;
    for (int j = 0; j < k; ++j)
        if (state[cn.regs[j]]) a |= 1ull << j;
    uint64_t q;
    double r;
    if (cn.kind == mbg::NODE_BINARY) {
        bool on = (cn.bits[a >> 5] >> (a & 31)) & 1u;
        q = on ? (state[node] ? cn.down : cn.up) : 0;
        r = on ? (state[node] ? cn.down_real : cn.up_real) : 0.0;
    } else {
        q = cn.palette[cn.pidx[a]];
        r = cn.palette_real[cn.pidx[a]];
    }
    if (fixed_rate) *fixed_rate = q;
    if (rate) *rate = r;
    return MBG_OK;
}

mbg_status mbg_model_with_rate_scales(const mbg_model* base, const double* up_scale, const double* down_scale,
                                      mbg_model** out) {
    if (!base || !out) return fail(MBG_ERR_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<mbg_model> m(new mbg_model());
    mbg_status st = guard([&] {
        m->cm = mbg::rescale_model(base->cm, up_scale, down_scale);
        m->names = base->names;
    });
    if (st != MBG_OK) return st;
    *out = m.release();
    return MBG_OK;
}

mbg_status mbg_model_with_mutations(const mbg_model* base, const int32_t* nodes, const int32_t* values,
                                    int32_t count, mbg_model** out) {
    if (!base || !out || (count > 0 && (!nodes || !values)) || count < 0) return fail(MBG_ERR_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<mbg_model> m(new mbg_model());
    mbg_status st = guard([&] {
        std::vector<int> nd(nodes, nodes + count), val(values, values + count);
        try {
            m->cm = mbg::mutate_model(base->cm, nd.data(), val.data(), count);
        } catch (const mbg::Error& e) {
            throw mbg::ModelError(e.what());
        }
        m->names = base->names;
    });
    if (st != MBG_OK) return st;
    *out = m.release();
    return MBG_OK;
}

mbg_status mbg_model_layout_check(const mbg_model* m) {
    if (!m) return fail(MBG_ERR_ARG, "null model");
    return guard([&] { mbg::check_layout(m->cm, mbg::layout_model(m->cm)); });
}

mbg_status mbg_model_jit_check(const mbg_model* m, double* compile_ms) {
    if (!m) return fail(MBG_ERR_ARG, "null model");
    return guard([&] {
        if (m->cm.words > 16) throw mbg::ModelError("thread layout supports at most 512 nodes");
        double ms = mbg::jit_compile_only(mbg::generate_thread_model(m->cm, mbg::layout_model(m->cm)));
        if (compile_ms) *compile_ms = ms;
    });
}

void mbg_sim_opts_default(mbg_sim_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->use_cfg_seed = 1;
    o->layout = MBG_LAYOUT_AUTO;
}

mbg_status mbg_sim_create(const mbg_model* m, const mbg_sim_opts* o, mbg_sim** out) {
    if (!m || !out) return fail(MBG_ERR_ARG, "null argument");
    *out = nullptr;
    mbg_sim_opts opts;
    if (o) opts = *o;
    else mbg_sim_opts_default(&opts);
    std::unique_ptr<mbg_sim> s(new mbg_sim());
    mbg_status st = guard([&] { s->sim.create(m->cm, m->names, opts); });
    if (st != MBG_OK) return st;
    *out = s.release();
    return MBG_OK;
}

void mbg_sim_destroy(mbg_sim* s) { delete s; }

mbg_status mbg_sim_run(mbg_sim* s, void* stream) {
    if (!s) return fail(MBG_ERR_ARG, "null simulation");
    return guard([&] { s->sim.run(static_cast<cudaStream_t>(stream)); });
}

mbg_status mbg_sim_summary(const mbg_sim* s, mbg_run_summary* out) {
    if (!s || !out) return fail(MBG_ERR_ARG, "null argument");
    if (!s->sim.ran) return fail(MBG_ERR_STATE, "summary requested before mbg_sim_run");
    *out = s->sim.summary;
    return MBG_OK;
}

mbg_status mbg_sim_probtraj(mbg_sim* s, double* probs, double* tr_entropy) {
    if (!s) return fail(MBG_ERR_ARG, "null simulation");
    return guard([&] {
        s->sim.fetch();
        if (probs) {
            std::memset(probs, 0, s->sim.n_bins * sizeof(double));
            for (size_t e = 0; e < s->sim.wbin.size(); ++e) probs[s->sim.wbin[e]] = mbg::window_prob(s->sim, s->sim.wsum[e]);
        }
        if (tr_entropy)
            for (int w = 0; w < s->sim.cm.windows; ++w) tr_entropy[w] = mbg::window_th(s->sim, w);
    });
}

mbg_status mbg_sim_probtraj_raw(mbg_sim* s, uint64_t* sums, uint64_t* th_sums) {
    if (!s) return fail(MBG_ERR_ARG, "null simulation");
    return guard([&] {
        s->sim.fetch();
        if (sums) {
            std::memset(sums, 0, s->sim.n_bins * 8);
            for (size_t e = 0; e < s->sim.wbin.size(); ++e) sums[s->sim.wbin[e]] = s->sim.wsum[e];
        }
        if (th_sums) std::memcpy(th_sums, s->sim.th.data(), s->sim.th.size() * 8);
    });
}

mbg_status mbg_sim_probtraj_sparse(mbg_sim* s, uint64_t* bins, uint64_t* sums, double* probs, size_t cap,
                                   size_t* count) {
    if (!s || !count) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        mbg::Sim& sim = s->sim;
        sim.fetch();
        const size_t n = sim.wbin.size();
        *count = n;
        const size_t m = n < cap ? n : cap;
        const uint32_t* wb = sim.wbin.data();
        const uint64_t* ws = sim.wsum.data();
        if (bins)
            for (size_t e = 0; e < m; ++e) bins[e] = wb[e];
        if (sums) std::memcpy(sums, ws, m * sizeof(uint64_t));
        if (probs) {
            // window_prob's arithmetic, in the same order (the dense read gives the same doubles)
            const double n_traj = (double)sim.n_traj;
            if (sim.cm.discrete) {
                for (size_t e = 0; e < m; ++e) probs[e] = (double)ws[e] / n_traj;
            } else {
                const double denom = n_traj * sim.cm.tick;
                for (size_t e = 0; e < m; ++e) probs[e] = ((double)ws[e] / 4294967296.0) / denom;
            }
        }
    });
}

mbg_status mbg_sim_final_states(mbg_sim* s, double* probs) {
    if (!s || !probs) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        const mbg::Sim& sim = s->sim;
        s->sim.fetch();
        const double n = (double)sim.n_traj;
        std::memset(probs, 0, sizeof(double) << sim.cm.n_out);
        for (size_t e = 0; e < sim.fin_state.size(); ++e) probs[sim.fin_state[e]] = (double)sim.fin_count[e] / n;
    });
}

mbg_status mbg_sim_final_states_sparse(mbg_sim* s, uint64_t* states, double* probs, size_t cap, size_t* count) {
    if (!s || !count) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        const mbg::Sim& sim = s->sim;
        s->sim.fetch();
        const size_t n = sim.fin_state.size();
        *count = n;
        const size_t m = n < cap ? n : cap;
        const double n_traj = (double)sim.n_traj;
        for (size_t e = 0; e < m; ++e) {
            if (states) states[e] = sim.fin_state[e];
            if (probs) probs[e] = (double)sim.fin_count[e] / n_traj;
        }
    });
}

mbg_status mbg_sim_fixed_points(mbg_sim* s, uint32_t* states, double* probs, size_t cap, size_t* count) {
    if (!s) return fail(MBG_ERR_ARG, "null simulation");
    return guard([&] {
        s->sim.fetch();
        const auto& f = s->sim.fixed;
        if (count) *count = f.size();
        const int W = s->sim.cm.words;
        for (size_t i = 0; i < f.size() && i < cap; ++i) {
            if (states) std::memcpy(states + i * W, f[i].words.data(), W * 4);
            if (probs) probs[i] = (double)f[i].count / (double)s->sim.n_traj;
        }
    });
}

mbg_status mbg_sim_trajectories(mbg_sim* s, uint32_t* states, double* times, uint32_t* transitions,
                                uint8_t* status) {
    if (!s) return fail(MBG_ERR_ARG, "null simulation");
    return guard([&] {
        mbg::Sim& x = s->sim;
        if (!x.ran) throw mbg::StateError("trajectories requested before mbg_sim_run");
        if (!x.prm.traj_state) throw mbg::StateError("record_trajectories was not set at create");
        cudaSetDevice(x.device);
        auto cp = [](void* dst, const void* src, size_t bytes) {
            cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) throw mbg::CudaError(std::string("cudaMemcpy D2H: ") + cudaGetErrorString(e));
        };
        if (states) cp(states, x.prm.traj_state, x.n_traj * x.cm.words * 4);
        if (times) cp(times, x.prm.traj_time, x.n_traj * 8);
        if (transitions) cp(transitions, x.prm.traj_transitions, x.n_traj * 4);
        if (status) cp(status, x.prm.traj_status, x.n_traj);
    });
}

mbg_status mbg_write_probtraj_csv(mbg_sim* s, const char* prefix) {
    if (!s || !prefix) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        s->sim.fetch();
        mbg::write_probtraj_csv(s->sim, std::string(prefix) + "_probtraj.csv");
    });
}

mbg_status mbg_write_fp_csv(mbg_sim* s, const char* prefix) {
    if (!s || !prefix) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        s->sim.fetch();
        mbg::write_fp_csv(s->sim, std::string(prefix) + "_fp.csv");
    });
}

mbg_status mbg_write_final_states_csv(mbg_sim* s, const char* prefix) {
    if (!s || !prefix) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        s->sim.fetch();
        mbg::write_final_states_csv(s->sim, std::string(prefix) + "_final_states.csv");
    });
}

mbg_status mbg_print_results(mbg_sim* s, const char* path) {
    if (!s || !path) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        s->sim.fetch();
        if (std::strcmp(path, "-") == 0) {
            mbg::print_results(s->sim, std::cout);
        } else {
            std::ofstream f(path);
            if (!f) throw mbg::IoError(std::string("cannot write ") + path);
            mbg::print_results(s->sim, f);
        }
    });
}


void mbg_batch_opts_default(mbg_batch_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
}

mbg_status mbg_batch_create(const mbg_model* const* models, int32_t n_models, const uint64_t* n_traj,
                            const uint64_t* seeds, const mbg_batch_opts* o, mbg_batch** out) {
    if (!models || n_models <= 0 || !out) return fail(MBG_ERR_ARG, "null or empty argument");
    *out = nullptr;
    mbg_batch_opts opts;
    if (o) opts = *o;
    else mbg_batch_opts_default(&opts);
    std::vector<const mbg::CompiledModel*> cms;
    for (int32_t i = 0; i < n_models; ++i) {
        if (!models[i]) return fail(MBG_ERR_ARG, "null model in batch");
        cms.push_back(&models[i]->cm);
    }
    std::vector<uint64_t> nt, sd;
    if (n_traj) nt.assign(n_traj, n_traj + n_models);
    if (seeds) sd.assign(seeds, seeds + n_models);
    std::unique_ptr<mbg_batch> b(new mbg_batch());
    mbg_status st = guard([&] { b->batch.create(cms, nt, sd, opts); });
    if (st != MBG_OK) return st;
    *out = b.release();
    return MBG_OK;
}

void mbg_batch_destroy(mbg_batch* b) { delete b; }

mbg_status mbg_batch_run(mbg_batch* b, void* stream) {
    if (!b) return fail(MBG_ERR_ARG, "null batch");
    return guard([&] { b->batch.run(static_cast<cudaStream_t>(stream)); });
}

mbg_status mbg_batch_summary(const mbg_batch* b, mbg_run_summary* out) {
    if (!b || !out) return fail(MBG_ERR_ARG, "null argument");
    if (!b->batch.ran) return fail(MBG_ERR_STATE, "summary requested before mbg_batch_run");
    *out = b->batch.summary;
    return MBG_OK;
}

mbg_status mbg_batch_instance_summary(const mbg_batch* b, int32_t i, mbg_run_summary* out) {
    if (!b || !out) return fail(MBG_ERR_ARG, "null argument");
    if (!b->batch.ran) return fail(MBG_ERR_STATE, "summary requested before mbg_batch_run");
    if (i < 0 || i >= (int32_t)b->batch.inst.size()) return fail(MBG_ERR_ARG, "instance index out of range");
    *out = b->batch.inst[i].summary;
    return MBG_OK;
}

mbg_status mbg_batch_probtraj(mbg_batch* b, int32_t i, double* probs, double* tr_entropy) {
    if (!b) return fail(MBG_ERR_ARG, "null batch");
    return guard([&] {
        b->batch.fetch(i);
        const mbg::Batch::Inst& x = b->batch.inst[i];
        const double n = (double)x.n_traj;
        const double tick = x.cm.tick;
        for (size_t k = 0; probs && k < x.hist.size(); ++k)
            probs[k] = x.cm.discrete ? (double)x.hist[k] / n : ((double)x.hist[k] / 4294967296.0) / (n * tick);
        for (int w = 0; tr_entropy && w < x.cm.windows; ++w) {
            double v = ((double)x.th[w] / 4294967296.0) / n;
            tr_entropy[w] = x.cm.discrete ? v : v / tick;
        }
    });
}

mbg_status mbg_batch_window_probs(mbg_batch* b, int32_t window, double* probs) {
    if (!b || !probs) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        std::vector<uint64_t> sums;
        b->batch.window_sums(window, sums);
        size_t o = 0;
        for (const mbg::Batch::Inst& x : b->batch.inst) {
            const size_t S = (size_t)1 << x.cm.n_out;
            const double n = (double)x.n_traj, tick = x.cm.tick;
            // mbg_batch_probtraj's arithmetic
            for (size_t k = 0; k < S; ++k)
                probs[o + k] = x.cm.discrete ? (double)sums[o + k] / n : ((double)sums[o + k] / 4294967296.0) / (n * tick);
            o += S;
        }
    });
}

mbg_status mbg_batch_probtraj_raw(mbg_batch* b, int32_t i, uint64_t* sums, uint64_t* th_sums) {
    if (!b) return fail(MBG_ERR_ARG, "null batch");
    return guard([&] {
        b->batch.fetch(i);
        const mbg::Batch::Inst& x = b->batch.inst[i];
        if (sums) std::memcpy(sums, x.hist.data(), x.hist.size() * 8);
        if (th_sums) std::memcpy(th_sums, x.th.data(), x.th.size() * 8);
    });
}

mbg_status mbg_batch_final_states(mbg_batch* b, int32_t i, double* probs) {
    if (!b || !probs) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        b->batch.fetch(i);
        const mbg::Batch::Inst& x = b->batch.inst[i];
        for (size_t k = 0; k < x.fin.size(); ++k) probs[k] = (double)x.fin[k] / (double)x.n_traj;
    });
}

mbg_status mbg_batch_fixed_points(mbg_batch* b, int32_t i, uint32_t* states, double* probs, size_t cap,
                                  size_t* count) {
    if (!b) return fail(MBG_ERR_ARG, "null batch");
    return guard([&] {
        b->batch.fetch(i);
        const mbg::Batch::Inst& x = b->batch.inst[i];
        const size_t W = (size_t)x.cm.words, nu = x.fp_cnt.size();
        // reference order: highest state word first (state.h:38-45)
        std::vector<size_t> order(nu);
        for (size_t k = 0; k < nu; ++k) order[k] = k;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t c) {
            for (size_t w = W; w-- > 0;)
                if (x.fp_words[a * W + w] != x.fp_words[c * W + w]) return x.fp_words[a * W + w] < x.fp_words[c * W + w];
            return false;
        });
        if (count) *count = nu;
        for (size_t k = 0; k < nu && k < cap; ++k) {
            if (states) std::memcpy(states + k * W, x.fp_words.data() + order[k] * W, W * 4);
            if (probs) probs[k] = (double)x.fp_cnt[order[k]] / (double)x.n_traj;
        }
    });
}

mbg_status mbg_surrogate_create(int32_t in_dim, int32_t hidden, int32_t hidden_layers, int32_t out_dim,
                                int32_t ensemble, uint64_t seed, int32_t device, mbg_surrogate** out) {
    if (!out) return fail(MBG_ERR_ARG, "null output pointer");
    *out = nullptr;
    std::unique_ptr<mbg_surrogate> s(new mbg_surrogate());
    mbg_status st = guard([&] {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            cudaGetLastError();
            throw mbg::CudaError("no CUDA device available");
        }
        if (device < 0 || device >= n) throw mbg::ArgError("device ordinal out of range");
        s->s.create(in_dim, hidden, hidden_layers, out_dim, ensemble, seed, device);
    });
    if (st != MBG_OK) return st;
    *out = s.release();
    return MBG_OK;
}

mbg_status mbg_surrogate_set_tensor_path(mbg_surrogate* s, int32_t tcgen05) {
    if (!s) return fail(MBG_ERR_ARG, "null surrogate");
    s->s.tensor_tc = tcgen05 != 0;
    return MBG_OK;
}

mbg_status mbg_surrogate_time_forward(mbg_surrogate* s, int32_t rows, int32_t reps, double* ms_per_pass) {
    if (!s || !ms_per_pass) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] { *ms_per_pass = s->s.time_forward(rows, reps); });
}

void mbg_surrogate_destroy(mbg_surrogate* s) { delete s; }

mbg_status mbg_surrogate_train(mbg_surrogate* s, const float* x, const float* y, int64_t n, int32_t epochs,
                               int32_t batch, float lr, uint64_t seed, float* last_loss) {
    if (!s || !x || !y) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] {
        float l = s->s.train(x, y, n, epochs, batch, lr, seed);
        if (last_loss) *last_loss = l;
    });
}

mbg_status mbg_surrogate_predict(mbg_surrogate* s, const float* x, int64_t n, float* probs, float* spread) {
    if (!s || !x) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] { s->s.predict(x, n, probs, spread); });
}

mbg_status mbg_surrogate_predict_column(mbg_surrogate* s, const float* x, int64_t n, int32_t column, float* score,
                                        float* spread) {
    if (!s || !x || !score) return fail(MBG_ERR_ARG, "null argument");
    return guard([&] { s->s.predict(x, n, nullptr, spread, column, score); });
}

int64_t mbg_surrogate_param_count(const mbg_surrogate* s) { return s ? s->s.param_count() : -1; }

mbg_status mbg_surrogate_get_params(mbg_surrogate* s, int32_t member, float* params) {
    if (!s || !params) return fail(MBG_ERR_ARG, "null argument");
    if (member < 0 || member >= s->s.ensemble) return fail(MBG_ERR_ARG, "ensemble member out of range");
    return guard([&] { s->s.get_params(member, params, false); });
}

mbg_status mbg_surrogate_set_params(mbg_surrogate* s, int32_t member, const float* params) {
    if (!s || !params) return fail(MBG_ERR_ARG, "null argument");
    if (member < 0 || member >= s->s.ensemble) return fail(MBG_ERR_ARG, "ensemble member out of range");
    return guard([&] { s->s.set_params(member, params); });
}

mbg_status mbg_surrogate_gradients(mbg_surrogate* s, int32_t member, const float* x, const float* y,
                                   int32_t rows, float* loss, float* grads) {
    if (!s || !x || !y || rows < 1) return fail(MBG_ERR_ARG, "null or empty argument");
    return guard([&] {
        float l = s->s.gradients(member, x, y, rows);
        if (loss) *loss = l;
        if (grads) s->s.get_params(member, grads, true);
    });
}

mbg_status mbg_batch_class_count(const mbg_batch* b, int32_t* count) {
    if (!b || !count) return fail(MBG_ERR_ARG, "null argument");
    *count = (int32_t)b->batch.classes.size();
    return MBG_OK;
}

mbg_status mbg_batch_class(const mbg_batch* b, int32_t c, mbg_batch_class_info* out) {
    if (!b || !out) return fail(MBG_ERR_ARG, "null argument");
    if (c < 0 || c >= (int32_t)b->batch.classes.size()) return fail(MBG_ERR_ARG, "class index out of range");
    const mbg::Batch::Class& k = b->batch.classes[c];
    *out = mbg_batch_class_info{};
    out->max_nodes = k.max_n;
    out->instances = (int32_t)k.members.size();
    out->trajectories = k.traj;
    out->layout = k.layout;
    out->block_size = k.block;
    out->variant = k.variant;
    out->grid = k.grid;
    out->kernel_ms = k.kernel_ms;
    out->timings = (int32_t)k.timings.size();
    return MBG_OK;
}

mbg_status mbg_batch_class_timings(const mbg_batch* b, int32_t c, mbg_batch_class_timing* out, int32_t cap,
                                   int32_t* count) {
    if (!b || !count || (cap > 0 && !out)) return fail(MBG_ERR_ARG, "null argument");
    if (c < 0 || c >= (int32_t)b->batch.classes.size()) return fail(MBG_ERR_ARG, "class index out of range");
    const auto& t = b->batch.classes[c].timings;
    *count = (int32_t)t.size();
    for (int32_t i = 0; i < cap && i < (int32_t)t.size(); ++i) out[i] = t[i];
    return MBG_OK;
}

}  // extern "C"
