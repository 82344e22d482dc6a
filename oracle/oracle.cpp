// Host FP64 Gillespie oracle: TEST INFRASTRUCTURE ONLY (see oracle.h for what it restates).
// The product never links this file, and this file uses nothing of the product: its parser,
// expression evaluation, random streams and fixed-point rules are its own (front.h).
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "front.h"

namespace {

using orc::Expr;
using orc::Op;

// Expression with node names and @aliases resolved for one node, as postfix instructions.
struct Prog {
    struct Ins {
        int code;  // 0 const, 1 node bit, 2 unary, 3 binary, 4 ternary
        double c;
        int node;
        Op op;
    };
    std::vector<Ins> ins;
};

void build(const Expr& e, const orc::ModelDef& m, int cur, Prog& p, int depth) {
    if (depth > 64) throw orc::Error("alias recursion too deep");
    switch (e.kind) {
        case Expr::Num: p.ins.push_back({0, e.value, 0, Op::Add}); break;
        case Expr::Var: {
            auto it = m.vars.find(e.name);
            if (it == m.vars.end()) throw orc::Error("unknown variable " + e.name);
            p.ins.push_back({0, it->second, 0, Op::Add});
            break;
        }
        case Expr::Node: {
            auto it = m.index.find(e.name);
            if (it == m.index.end()) throw orc::Error("unknown node name: " + e.name);
            p.ins.push_back({1, 0, it->second, Op::Add});
            break;
        }
        case Expr::Alias: {  // src/parser/expressions.cpp:223-231: the current node's attribute
            const Expr* a = m.nodes[cur].attr(e.name.substr(1));
            if (!a) throw orc::Error("missing attribute " + e.name);
            build(*a, m, cur, p, depth + 1);
            break;
        }
        case Expr::Unary:
            build(*e.a, m, cur, p, depth);
            p.ins.push_back({2, 0, 0, e.op});
            break;
        case Expr::Binary:
            build(*e.a, m, cur, p, depth);
            build(*e.b, m, cur, p, depth);
            p.ins.push_back({3, 0, 0, e.op});
            break;
        case Expr::Ternary:
            build(*e.a, m, cur, p, depth);
            build(*e.b, m, cur, p, depth);
            build(*e.c, m, cur, p, depth);
            p.ins.push_back({4, 0, 0, Op::Add});
            break;
    }
}

double run(const Prog& p, const uint8_t* s, double* st) {
    int sp = 0;
    for (const auto& in : p.ins) {
        switch (in.code) {
            case 0: st[sp++] = in.c; break;
            case 1: st[sp++] = s[in.node] ? 1.0 : 0.0; break;
            case 2: st[sp - 1] = orc::apply(in.op, 0, st[sp - 1]); break;
            case 3:
                st[sp - 2] = orc::apply(in.op, st[sp - 2], st[sp - 1]);
                --sp;
                break;
            case 4: {
                double c = st[sp - 3];
                st[sp - 3] = c != 0 ? st[sp - 2] : st[sp - 1];
                sp -= 2;
                break;
            }
        }
    }
    return st[0];
}

struct Local {
    std::unordered_map<uint64_t, double> hist;
    std::vector<double> th, fin;
    uint64_t cnt[7] = {0, 0, 0, 0, 0, 0, 0};
};

}  // namespace

struct orc_result {
    int n = 0, words = 0, n_out = 0, windows = 0, threads = 1;
    bool discrete = false;
    uint64_t n_traj = 0;
    std::map<uint64_t, double> hist;  // (window << 32 | state) -> value
    std::vector<double> th, fin;
    uint64_t cnt[7] = {0, 0, 0, 0, 0, 0, 0};
    std::vector<uint32_t> states;
    std::vector<double> times;
    std::vector<uint32_t> trans;
    std::vector<uint8_t> status, ties;
    double seconds = 0;
};

extern "C" orc_result* orc_run(const char* bnd_text, const char* cfg_text, const orc_opts* o, char* err,
                               size_t errlen) {
    try {
        orc::ModelDef m;
        orc::parse_model(m, bnd_text, cfg_text);
        const int n = (int)m.nodes.size();
        if (n == 0) throw orc::Error("model has no nodes");
        auto* res = new orc_result();
        res->n = n;
        res->words = (n + 31) / 32;
        std::vector<int> out_nodes;
        for (int i = 0; i < n; ++i)
            if (!orc::is_internal(m, i)) out_nodes.push_back(i);
        res->n_out = (int)out_nodes.size();
        if (res->n_out > 24) throw orc::Error("too many output nodes for the oracle");
        const bool discrete = m.constant("discrete_time") != 0;
        const double max_time = m.constant("max_time"), tick = m.constant("time_tick");
        res->discrete = discrete;
        res->windows = std::max(1, (int)std::ceil((float)max_time / (float)tick));
        const int K = res->windows;
        const uint64_t S = 1ull << res->n_out;
        double sc = m.constant("sample_count");
        res->n_traj = o->n_traj ? o->n_traj : (uint64_t)(sc > 0 ? sc : 0);
        double cs = m.constant("seed_pseudorandom");
        const uint64_t seed = o->use_cfg_seed ? (uint64_t)(cs > 0 ? cs : 0) : o->seed;
        const uint32_t max_steps = o->max_steps;

        std::vector<Prog> up(n), down(n);
        std::vector<uint32_t> thr(n);
        for (int i = 0; i < n; ++i) {
            build(*m.nodes[i].attr("rate_up"), m, i, up[i], 0);
            build(*m.nodes[i].attr("rate_down"), m, i, down[i], 0);
            thr[i] = (uint32_t)std::floor(m.nodes[i].istate * 16777216.0);
        }
        size_t depth = 0;
        for (int i = 0; i < n; ++i) depth = std::max({depth, up[i].ins.size(), down[i].ins.size()});
        // the pick's fixed-point scale: the caller's, or the rule of the simulator (every node's
        // largest rate over all states of the nodes its rates read, summed)
        int F = o->frac_bits;
        if (F <= 0) {
            std::vector<uint8_t> st(n, 0);
            std::vector<double> stack(depth + 2);
            double sum_max = 0;
            for (int i = 0; i < n; ++i) {
                std::vector<int> sup{i};
                for (const Prog* pg : {&up[i], &down[i]})
                    for (const auto& in : pg->ins)
                        if (in.code == 1 && std::find(sup.begin(), sup.end(), in.node) == sup.end()) sup.push_back(in.node);
                if (sup.size() > 26) throw orc::Error("a rate reads more than 25 other nodes");
                double mx = 0;
                for (uint64_t a = 0; a < (1ull << sup.size()); ++a) {
                    for (size_t q = 0; q < sup.size(); ++q) st[sup[q]] = (uint8_t)((a >> q) & 1u);
                    mx = std::max(mx, run(st[i] ? down[i] : up[i], st.data(), stack.data()));
                }
                for (int x : sup) st[x] = 0;
                sum_max += mx;
            }
            F = orc::frac_bits_for(sum_max);
        }

        int T = o->threads > 0 ? o->threads : (int)std::thread::hardware_concurrency();
        if (T < 1) T = 1;
        if ((uint64_t)T > res->n_traj) T = (int)std::max<uint64_t>(1, res->n_traj);
        res->threads = T;
        const bool keep = o->keep_trajectories != 0;
        const int W = res->words;
        if (keep) {
            res->states.assign(res->n_traj * W, 0);
            res->times.assign(res->n_traj, 0);
            res->trans.assign(res->n_traj, 0);
            res->status.assign(res->n_traj, 0);
            res->ties.assign(res->n_traj, 0);
        }
        std::vector<Local> locals(T);
        std::atomic<uint64_t> next{0};
        const double two64 = 18446744073709551616.0;

        auto worker = [&](int tid) {
            Local& L = locals[tid];
            L.th.assign(K, 0.0);
            L.fin.assign(S, 0.0);
            std::vector<uint8_t> s(n);
            std::vector<double> r(n), stack(depth + 2);
            std::vector<uint64_t> q(n);
            auto add_slice = [&](double t0, double t1, uint32_t so, double h) {
                if (!(t1 > t0)) return;
                int w = (int)std::floor(t0 / tick);
                while (t1 > t0) {
                    double wend = (w + 1) * tick;
                    double len = std::min(t1, wend) - t0;
                    int wc = std::min(std::max(w, 0), K - 1);
                    L.hist[((uint64_t)wc << 32) | so] += len;
                    L.th[wc] += h * len;
                    ++w;
                    t0 = std::min(t1, wend);
                }
            };
            for (;;) {
                uint64_t j = next.fetch_add(1);
                if (j >= res->n_traj) break;
                const uint64_t traj = o->traj_base + j;
                for (int b = 0; 4 * b < n; ++b) {
                    orc::W4 d = orc::init_draws(seed, traj, (uint32_t)b);
                    unsigned w4[4] = {d.x, d.y, d.z, d.w};
                    for (int c = 0; c < 4 && 4 * b + c < n; ++c) s[4 * b + c] = (w4[c] >> 8) < thr[4 * b + c];
                }
                double t = 0;
                uint64_t step = 0;
                uint32_t trans = 0;
                uint8_t status = 0, tie = 0;
                int legacy_flip = -1;
                for (;;) {
                    uint64_t Q = 0;
                    double R = 0, Rout = 0;
                    for (int i = 0; i < n; ++i) {
                        r[i] = run(s[i] ? down[i] : up[i], s.data(), stack.data());
                        q[i] = orc::quantize(r[i], F);
                        Q += q[i];
                        R += r[i];
                    }
                    uint32_t so = 0;
                    for (size_t p = 0; p < out_nodes.size(); ++p) {
                        so |= (uint32_t)s[out_nodes[p]] << p;
                        Rout += r[out_nodes[p]];
                    }
                    if (Q == 0) {  // fixed point: the state holds until max_time
                        if (discrete) {
                            int w = std::min((int)step, K - 1);
                            L.hist[((uint64_t)w << 32) | so] += 1.0;
                        } else {
                            add_slice(t, max_time, so, 0.0);
                        }
                        t = max_time;
                        status = orc::FIXED_POINT;
                        break;
                    }
                    if (max_steps && step >= max_steps) {
                        status = orc::STEP_LIMIT;
                        break;
                    }
                    double h = 0;
                    if (Rout > 0)
                        for (int p : out_nodes) {
                            double pr = r[p] / Rout;
                            if (pr != 0) h -= std::log2(pr) * pr;
                        }
                    orc::W4 d = orc::step_draws(seed, traj, step);
                    double t1;
                    if (discrete) {
                        t1 = (double)(step + 1) * tick;
                        if (step + 1 >= (uint64_t)K) t1 = max_time;
                        int w = std::min((int)step, K - 1);
                        L.hist[((uint64_t)w << 32) | so] += 1.0;
                        L.th[w] += h;
                    } else {
                        double dt = -std::log(orc::unit_open0(d.x)) / R;
                        t1 = t + dt;
                        if (std::fabs(t1 - max_time) <= 1e-6 * max_time) tie |= 2;
                        t1 = std::min(t1, max_time);
                        add_slice(t, t1, so, h);
                    }
                    if (t1 >= max_time) {
                        t = max_time;
                        status = orc::FINISHED;
                        if (o->legacy_final) {
                            uint64_t rt = orc::pick_target(d.y, d.z, Q), acc = 0;
                            for (int i = 0; i < n; ++i) {
                                acc += q[i];
                                if (acc > rt) {
                                    legacy_flip = i;
                                    break;
                                }
                            }
                        }
                        break;
                    }
                    if (o->redraw_period && (step + 1) % o->redraw_period == 0) {
                        // the reference's launch segments (simulation_runner.cu:51 with
                        // simulation.cu:143-147): the segment's last record ends without a flip and
                        // the next launch draws the holding time of the same state again
                        t = t1;
                        ++step;
                        continue;
                    }
                    uint64_t rt = orc::pick_target(d.y, d.z, Q);
                    uint64_t acc = 0;
                    int k = -1;
                    for (int i = 0; i < n; ++i) {
                        acc += q[i];
                        if (acc > rt) {
                            k = i;
                            break;
                        }
                    }
                    double u = ((double)(((uint64_t)d.y << 32) | d.z)) / two64;
                    double rr = u * R, ar = 0;
                    int kk = n - 1;
                    for (int i = 0; i < n; ++i) {
                        ar += r[i];
                        if (ar > rr) {
                            kk = i;
                            break;
                        }
                    }
                    if (kk != k) tie |= 1;
                    if (k < 0) {
                        status = orc::FAILED;
                        break;
                    }
                    s[k] ^= 1;
                    t = t1;
                    ++step;
                    ++trans;
                }
                uint32_t so = 0;
                if (legacy_flip >= 0) s[legacy_flip] ^= 1;
                for (size_t p = 0; p < out_nodes.size(); ++p) so |= (uint32_t)s[out_nodes[p]] << p;
                if (legacy_flip >= 0) s[legacy_flip] ^= 1;
                L.cnt[0] += trans;
                L.cnt[6] += step + (status == orc::STEP_LIMIT ? 0 : 1);
                if (status == orc::FINISHED) ++L.cnt[1];
                if (status == orc::FIXED_POINT) ++L.cnt[2];
                if (status == orc::STEP_LIMIT) ++L.cnt[3];
                if (tie & 1) ++L.cnt[4];
                if (tie & 2) ++L.cnt[5];
                if (status == orc::FINISHED || status == orc::FIXED_POINT) L.fin[so] += 1.0;
                if (keep) {
                    for (int w = 0; w < W; ++w) {
                        uint32_t word = 0;
                        for (int b = 0; b < 32 && 32 * w + b < n; ++b) word |= (uint32_t)s[32 * w + b] << b;
                        res->states[j * W + w] = word;
                    }
                    res->times[j] = t;
                    res->trans[j] = trans;
                    res->status[j] = status;
                    res->ties[j] = tie;
                }
            }
        };
        auto t0 = std::chrono::steady_clock::now();
        std::vector<std::thread> pool;
        for (int i = 1; i < T; ++i) pool.emplace_back(worker, i);
        worker(0);
        for (auto& th : pool) th.join();
        res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        res->th.assign(K, 0.0);
        res->fin.assign(S, 0.0);
        for (auto& L : locals) {
            for (auto& kv : L.hist) res->hist[kv.first] += kv.second;
            for (int w = 0; w < K; ++w) res->th[w] += L.th[w];
            for (uint64_t x = 0; x < S; ++x) res->fin[x] += L.fin[x];
            for (int c = 0; c < 7; ++c) res->cnt[c] += L.cnt[c];
        }
        return res;
    } catch (const std::exception& e) {
        if (err && errlen) {
            std::strncpy(err, e.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return nullptr;
    }
}

extern "C" void orc_free(orc_result* r) { delete r; }

extern "C" void orc_dims(const orc_result* r, int* n, int* words, int* n_out, int* windows) {
    *n = r->n;
    *words = r->words;
    *n_out = r->n_out;
    *windows = r->windows;
}

extern "C" void orc_counters(const orc_result* r, uint64_t* out7) {
    for (int i = 0; i < 7; ++i) out7[i] = r->cnt[i];
}

extern "C" size_t orc_hist_nnz(const orc_result* r) { return r->hist.size(); }

extern "C" void orc_hist_get(const orc_result* r, uint32_t* window, uint32_t* state, double* value) {
    size_t i = 0;
    for (auto& kv : r->hist) {
        window[i] = (uint32_t)(kv.first >> 32);
        state[i] = (uint32_t)kv.first;
        value[i] = kv.second;
        ++i;
    }
}

extern "C" void orc_th(const orc_result* r, double* th) { std::copy(r->th.begin(), r->th.end(), th); }

extern "C" void orc_final(const orc_result* r, double* counts) { std::copy(r->fin.begin(), r->fin.end(), counts); }

extern "C" void orc_trajectories(const orc_result* r, uint32_t* states, double* times, uint32_t* transitions,
                                 uint8_t* status, uint8_t* ties) {
    if (r->states.empty()) return;
    if (states) std::copy(r->states.begin(), r->states.end(), states);
    if (times) std::copy(r->times.begin(), r->times.end(), times);
    if (transitions) std::copy(r->trans.begin(), r->trans.end(), transitions);
    if (status) std::copy(r->status.begin(), r->status.end(), status);
    if (ties) std::copy(r->ties.begin(), r->ties.end(), ties);
}

extern "C" double orc_seconds(const orc_result* r) { return r->seconds; }
extern "C" int orc_threads(const orc_result* r) { return r->threads; }

extern "C" void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    const orc::W4 d = orc::philox10({ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
    out[0] = d.x;
    out[1] = d.y;
    out[2] = d.z;
    out[3] = d.w;
}
