// Source generator for the per-model thread-per-trajectory evaluator compiled by NVRTC.
//
// The reference emits one `<node>_rate(state)` function per node plus an aggregate that writes
// all N rates to a thread-local array (src/generator.cpp:84-144) and scans that array to pick a
// node (src/jit_kernels/simulation.cu:9-21). Here the generated code keeps everything in
// registers: pass 1 evaluates every node from its truth table (a literal for up to 6 table bits)
// and keeps one "active" bit per node plus the exact fixed-point total; pass 2 re-derives each
// active node's rate from the active and state bits and counts prefixes at or below the target.
// A model whose nodes all share one rate skips pass 2's arithmetic: the pick is the m-th active
// bit with m = r / rate.
#include <cmath>
#include <cstdio>
#include <sstream>

#include "model.hpp"
#include "sim_host.hpp"

namespace mbg {

namespace {

std::string u64lit(uint64_t v) { return std::to_string(v) + "ull"; }

std::string flit(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%.9ef", v);
    return b;
}

std::string bit_expr(int i) {
    return "((s[" + std::to_string(i >> 5) + "] >> " + std::to_string(i & 31) + ") & 1u)";
}

std::string act_expr(int i) {
    return "((act[" + std::to_string(i >> 5) + "] >> " + std::to_string(i & 31) + ") & 1u)";
}

// x = (self << k) | regulator bits
std::string index_expr(const CompiledNode& cn, int i) {
    std::ostringstream o;
    int k = (int)cn.regs.size();
    o << "(" << bit_expr(i) << " << " << k << ")";
    for (int j = 0; j < k; ++j) o << " | (" << bit_expr(cn.regs[j]) << " << " << j << ")";
    return o.str();
}

std::string table_bit_expr(const CompiledNode& cn, const DeviceLayout& dl, int i) {
    int k = (int)cn.regs.size();
    std::ostringstream o;
    if (k + 1 <= 5) {
        o << "((" << cn.bits[0] << "u >> x) & 1u)";
    } else if (k + 1 == 6) {
        uint64_t t = (uint64_t)cn.bits[0] | ((uint64_t)cn.bits[1] << 32);
        o << "((unsigned)(" << u64lit(t) << " >> x) & 1u)";
    } else {
        o << "((__ldg(p.tabs + " << dl.tab_off[i] << "u + (x >> 5)) >> (x & 31u)) & 1u)";
    }
    return o.str();
}

double rlog2r(double r) { return r > 0 ? r * std::log2(r) : 0.0; }

}  // namespace

std::string generate_thread_model(const CompiledModel& cm, const DeviceLayout& dl) {
    const int W = cm.words;
    bool uniform = true;
    uint64_t urate = 0;
    for (int i = 0; i < cm.n; ++i) {
        const CompiledNode& cn = cm.nodes[i];
        if (cn.kind != NODE_BINARY || cn.up != cn.down || cn.up == 0) {
            uniform = false;
            break;
        }
        if (i == 0) urate = cn.up;
        if (cn.up != urate) {
            uniform = false;
            break;
        }
    }
    std::ostringstream o;
    o << "namespace mbg {\nstruct JitModel {\n  static constexpr int W = " << W << ";\n";

    // ---- pass 1
    o << "  __device__ __forceinline__ static unsigned long long eval(const SimParams& p, const unsigned (&s)[W], "
         "unsigned (&act)[W], unsigned long long& rout, float& cout) {\n";
    o << "    unsigned long long t = 0ull, ro = 0ull; float co = 0.f;\n";
    for (int w = 0; w < W; ++w) o << "    unsigned a" << w << " = 0u;\n";
    for (int i = 0; i < cm.n; ++i) {
        const CompiledNode& cn = cm.nodes[i];
        const bool out = cm.out_pos[i] >= 0;
        o << "    { const unsigned x = " << index_expr(cn, i) << ";\n";
        if (cn.kind == NODE_BINARY) {
            o << "      const unsigned on = " << table_bit_expr(cn, dl, i) << ";\n";
            o << "      a" << (i >> 5) << " |= on << " << (i & 31) << ";\n";
            if (!uniform || out) {
                std::string sel = cn.up == cn.down ? u64lit(cn.up)
                                                   : "(" + bit_expr(i) + " ? " + u64lit(cn.down) + " : " +
                                                         u64lit(cn.up) + ")";
                o << "      const unsigned long long r = on ? " << sel << " : 0ull;\n";
                if (!uniform) o << "      t += r;\n";
                if (out) {
                    o << "      ro += r;\n";
                    double cu = rlog2r(cn.up_real), cd = rlog2r(cn.down_real);
                    if (cu != 0 || cd != 0)
                        o << "      co += on ? (" << bit_expr(i) << " ? " << flit(cd) << " : " << flit(cu)
                          << ") : 0.f;\n";
                }
            }
        } else {
            o << "      const unsigned long long r = __ldg(p.palette + " << dl.pal_off[i]
              << "u + __ldg(p.pidx + " << dl.tab_off[i] << "u + x));\n";
            o << "      a" << (i >> 5) << " |= (unsigned)(r != 0ull) << " << (i & 31) << ";\n";
            o << "      t += r;\n";
            if (out)
                o << "      ro += r; if (r) { const float rr = (float)r * p.to_real; co += rr * __log2f(rr); }\n";
        }
        o << "    }\n";
    }
    if (uniform) {
        o << "    t = (unsigned long long)(0";
        for (int w = 0; w < W; ++w) o << " + __popc(a" << w << ")";
        o << ") * " << u64lit(urate) << ";\n";
    }
    for (int w = 0; w < W; ++w) o << "    act[" << w << "] = a" << w << ";\n";
    o << "    rout = ro; cout = co; return t;\n  }\n";

    // ---- pass 2
    o << "  __device__ __forceinline__ static int pick(const SimParams& p, const unsigned (&s)[W], "
         "const unsigned (&act)[W], unsigned long long r) {\n";
    if (uniform) {
        o << "    unsigned m = (unsigned)(r / " << u64lit(urate) << ");\n";
        for (int w = 0; w < W; ++w) {
            o << "    { const unsigned c = __popc(act[" << w << "]); if (m < c) return " << 32 * w
              << " + (int)__fns(act[" << w << "], 0u, (int)m + 1); m -= c; }\n";
        }
        o << "    return -1;\n  }\n";
    } else {
        o << "    unsigned long long acc = 0ull; int c = 0;\n";
        for (int i = 0; i < cm.n; ++i) {
            const CompiledNode& cn = cm.nodes[i];
            if (cn.kind == NODE_BINARY) {
                if (cn.up == 0 && cn.down == 0) {
                    o << "    c += acc <= r;\n";
                    continue;
                }
                std::string sel = cn.up == cn.down ? u64lit(cn.up)
                                                   : "(" + bit_expr(i) + " ? " + u64lit(cn.down) + " : " +
                                                         u64lit(cn.up) + ")";
                o << "    acc += " << act_expr(i) << " ? " << sel << " : 0ull; c += acc <= r;\n";
            } else {
                o << "    { const unsigned x = " << index_expr(cn, i) << "; acc += __ldg(p.palette + "
                  << dl.pal_off[i] << "u + __ldg(p.pidx + " << dl.tab_off[i] << "u + x)); c += acc <= r; }\n";
            }
        }
        o << "    return c;\n  }\n";
    }

    // ---- output index (get_non_internal_index, generator.cpp:207-235)
    o << "  __device__ __forceinline__ static unsigned out_index(const SimParams& p, const unsigned (&s)[W]) {\n";
    o << "    return 0u";
    for (int q = 0; q < cm.n_out; ++q) o << " | (" << bit_expr(cm.out_nodes[q]) << " << " << q << ")";
    o << ";\n  }\n};\n}  // namespace mbg\n";
    o << "extern \"C\" __global__ void __launch_bounds__(256) mbg_sim_thread(const mbg::SimParams p) {\n"
         "  mbg::sim_thread_body<mbg::JitModel>(p);\n}\n";
    return o.str();
}

}  // namespace mbg
