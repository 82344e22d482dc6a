// Expression evaluation and compilation of a parsed model into per-node rate tables.
//
// Rate semantics restate src/generator.cpp:84-122: a node's rate is `rate_down` when the node is
// on and `rate_up` when it is off, with @aliases resolved against the node's own attributes
// (src/parser/expressions.cpp:223-231). The `@logic ? x : 0` fast path of generator.cpp:93-107
// is the same function and needs no special case here: every node is tabulated over its
// regulators instead of being emitted as source text.
#include <algorithm>
#include <thread>
#include <mutex>
#include <exception>
#include <atomic>
#include <cmath>
#include <cstring>
#include <set>

#include "model.hpp"
#include "parallel.hpp"

namespace mbg {

const Expr* Node::attr(const std::string& n) const {
    for (auto& a : attrs)
        if (a.first == n) return a.second.get();
    return nullptr;
}

Model::Model() {
    constants["discrete_time"] = 0;
    constants["sample_count"] = 1000000;
    constants["max_time"] = 10;
    constants["time_tick"] = 0.1;
    constants["seed_pseudorandom"] = 0;
}

int Model::node_index(const std::string& name) const {
    auto it = index.find(name);
    return it == index.end() ? -1 : it->second;
}

void Model::add_node(Node&& n) {
    index.emplace(n.name, (int)nodes.size());
    nodes.push_back(std::move(n));
}

double Model::constant(const std::string& n) const {
    auto it = constants.find(n);
    return it == constants.end() ? 0.0 : it->second;
}

bool Model::is_internal(int i) const {
    const Expr* e = nodes[i].attr("is_internal");
    return e && eval_const(*e, *this) != 0;
}

static double apply_unary(Op op, double x) {
    switch (op) {
        case Op::Plus: return x;
        case Op::Minus: return -x;
        case Op::Not: return x == 0 ? 1.0 : 0.0;
        default: throw Error("Unknown unary operator");
    }
}

static double apply_binary(Op op, double l, double r) {
    switch (op) {
        case Op::Plus: return l + r;
        case Op::Minus: return l - r;
        case Op::Star: return l * r;
        case Op::Slash: return l / r;
        case Op::And: return (l != 0 && r != 0) ? 1.0 : 0.0;
        case Op::Or: return (l != 0 || r != 0) ? 1.0 : 0.0;
        case Op::Xor: return ((l != 0) != (r != 0)) ? 1.0 : 0.0;
        case Op::Eq: return l == r ? 1.0 : 0.0;
        case Op::Ne: return l != r ? 1.0 : 0.0;
        case Op::Le: return l <= r ? 1.0 : 0.0;
        case Op::Lt: return l < r ? 1.0 : 0.0;
        case Op::Ge: return l >= r ? 1.0 : 0.0;
        case Op::Gt: return l > r ? 1.0 : 0.0;
        default: throw Error("Unknown binary operator");
    }
}

static double lookup_var(const Model& m, const std::string& name) {
    auto it = m.variables.find(name);
    if (it == m.variables.end()) throw Error("unknown variable " + name);
    return it->second;
}

double eval_const(const Expr& e, const Model& m) {
    switch (e.kind) {
        case Expr::Kind::Literal: return e.value;
        case Expr::Kind::Ident: throw Error("identifier " + e.name + " in expression which needs to be evaluated");
        case Expr::Kind::Var: return lookup_var(m, e.name);
        case Expr::Kind::Alias: throw Error("alias " + e.name + " in expression which needs to be evaluated");
        case Expr::Kind::Unary: return apply_unary(e.op, eval_const(*e.a, m));
        case Expr::Kind::Binary: return apply_binary(e.op, eval_const(*e.a, m), eval_const(*e.b, m));
        case Expr::Kind::Ternary: return eval_const(*e.a, m) != 0 ? eval_const(*e.b, m) : eval_const(*e.c, m);
        case Expr::Kind::Paren: return eval_const(*e.a, m);
    }
    return 0;
}

static const Expr& resolve_alias(const Expr& e, const Model& m, int cur) {
    const Expr* a = m.nodes[cur].attr(e.name.substr(1));
    if (!a) throw Error("Node " + m.nodes[cur].name + " does not have attribute " + e.name.substr(1));
    return *a;
}

double eval_state(const Expr& e, const Model& m, int cur, const uint8_t* state) {
    switch (e.kind) {
        case Expr::Kind::Literal: return e.value;
        case Expr::Kind::Ident: {
            int i = m.node_index(e.name);
            if (i < 0) throw Error("unknown node name: " + e.name);
            return state[i] ? 1.0 : 0.0;
        }
        case Expr::Kind::Var: return lookup_var(m, e.name);
        case Expr::Kind::Alias: return eval_state(resolve_alias(e, m, cur), m, cur, state);
        case Expr::Kind::Unary: return apply_unary(e.op, eval_state(*e.a, m, cur, state));
        case Expr::Kind::Binary:
            return apply_binary(e.op, eval_state(*e.a, m, cur, state), eval_state(*e.b, m, cur, state));
        case Expr::Kind::Ternary:
            return eval_state(*e.a, m, cur, state) != 0 ? eval_state(*e.b, m, cur, state)
                                                         : eval_state(*e.c, m, cur, state);
        case Expr::Kind::Paren: return eval_state(*e.a, m, cur, state);
    }
    return 0;
}

void collect_support(const Expr& e, const Model& m, int cur, std::vector<int>& out, int depth) {
    if (depth > 64) throw Error("alias recursion too deep in node " + m.nodes[cur].name);
    switch (e.kind) {
        case Expr::Kind::Ident: {
            int i = m.node_index(e.name);
            if (i < 0) throw Error("unknown node name: " + e.name);
            out.push_back(i);
            break;
        }
        case Expr::Kind::Alias: collect_support(resolve_alias(e, m, cur), m, cur, out, depth + 1); break;
        default:
            if (e.a) collect_support(*e.a, m, cur, out, depth);
            if (e.b) collect_support(*e.b, m, cur, out, depth);
            if (e.c) collect_support(*e.c, m, cur, out, depth);
    }
}

// ---------------------------------------------------------------------------------------------
// Block evaluator: an expression flattened to postfix form over "input bits" (the node's
// regulators, then the node itself), evaluated for 64 assignments at a time. Tabulating a node
// with k regulators costs 2^(k+1) evaluations, so this matters for hub nodes.

namespace {

constexpr int kBlock = 64;

struct Instr {
    enum Code { Const, Bit, Un, Bin, Tern } code;
    double c = 0;
    int bit = 0;
    Op op = Op::Plus;
};

void flatten(const Expr& e, const Model& m, int cur, const std::vector<int>& inputs, std::vector<Instr>& prog,
             int depth) {
    if (depth > 64) throw Error("alias recursion too deep in node " + m.nodes[cur].name);
    switch (e.kind) {
        case Expr::Kind::Literal: prog.push_back({Instr::Const, e.value}); break;
        case Expr::Kind::Var: prog.push_back({Instr::Const, lookup_var(m, e.name)}); break;
        case Expr::Kind::Ident: {
            int i = m.node_index(e.name);
            auto it = std::find(inputs.begin(), inputs.end(), i);
            if (it == inputs.end()) throw Error("internal: node outside support");
            Instr in{Instr::Bit};
            in.bit = (int)(it - inputs.begin());
            prog.push_back(in);
            break;
        }
        case Expr::Kind::Alias: flatten(resolve_alias(e, m, cur), m, cur, inputs, prog, depth + 1); break;
        case Expr::Kind::Paren: flatten(*e.a, m, cur, inputs, prog, depth); break;
        case Expr::Kind::Unary: {
            flatten(*e.a, m, cur, inputs, prog, depth);
            Instr in{Instr::Un};
            in.op = e.op;
            prog.push_back(in);
            break;
        }
        case Expr::Kind::Binary: {
            flatten(*e.a, m, cur, inputs, prog, depth);
            flatten(*e.b, m, cur, inputs, prog, depth);
            Instr in{Instr::Bin};
            in.op = e.op;
            prog.push_back(in);
            break;
        }
        case Expr::Kind::Ternary:
            flatten(*e.a, m, cur, inputs, prog, depth);
            flatten(*e.b, m, cur, inputs, prog, depth);
            flatten(*e.c, m, cur, inputs, prog, depth);
            prog.push_back({Instr::Tern});
            break;
    }
}

// Evaluates `prog` for assignments a0 .. a0+63, input bit j = (a >> j) & 1.
void run_block(const std::vector<Instr>& prog, uint64_t a0, std::vector<double>& stack, double* out) {
    size_t sp = 0;
    for (const Instr& in : prog) {
        switch (in.code) {
            case Instr::Const: {
                double* d = &stack[sp++ * kBlock];
                for (int t = 0; t < kBlock; ++t) d[t] = in.c;
                break;
            }
            case Instr::Bit: {
                double* d = &stack[sp++ * kBlock];
                for (int t = 0; t < kBlock; ++t) d[t] = (double)(((a0 + t) >> in.bit) & 1u);
                break;
            }
            case Instr::Un: {
                double* d = &stack[(sp - 1) * kBlock];
                switch (in.op) {
                    case Op::Plus: break;
                    case Op::Minus: for (int t = 0; t < kBlock; ++t) d[t] = -d[t]; break;
                    case Op::Not: for (int t = 0; t < kBlock; ++t) d[t] = d[t] == 0 ? 1.0 : 0.0; break;
                    default: for (int t = 0; t < kBlock; ++t) d[t] = apply_unary(in.op, d[t]); break;
                }
                break;
            }
            case Instr::Bin: {
                // one loop per operator (apply_binary's rules), so that each loop vectorises
                double* l = &stack[(sp - 2) * kBlock];
                const double* r = &stack[(sp - 1) * kBlock];
                switch (in.op) {
                    case Op::Plus: for (int t = 0; t < kBlock; ++t) l[t] = l[t] + r[t]; break;
                    case Op::Minus: for (int t = 0; t < kBlock; ++t) l[t] = l[t] - r[t]; break;
                    case Op::Star: for (int t = 0; t < kBlock; ++t) l[t] = l[t] * r[t]; break;
                    case Op::Slash: for (int t = 0; t < kBlock; ++t) l[t] = l[t] / r[t]; break;
                    case Op::And: for (int t = 0; t < kBlock; ++t) l[t] = (l[t] != 0 && r[t] != 0) ? 1.0 : 0.0; break;
                    case Op::Or: for (int t = 0; t < kBlock; ++t) l[t] = (l[t] != 0 || r[t] != 0) ? 1.0 : 0.0; break;
                    case Op::Xor: for (int t = 0; t < kBlock; ++t) l[t] = ((l[t] != 0) != (r[t] != 0)) ? 1.0 : 0.0; break;
                    case Op::Eq: for (int t = 0; t < kBlock; ++t) l[t] = l[t] == r[t] ? 1.0 : 0.0; break;
                    case Op::Ne: for (int t = 0; t < kBlock; ++t) l[t] = l[t] != r[t] ? 1.0 : 0.0; break;
                    case Op::Le: for (int t = 0; t < kBlock; ++t) l[t] = l[t] <= r[t] ? 1.0 : 0.0; break;
                    case Op::Lt: for (int t = 0; t < kBlock; ++t) l[t] = l[t] < r[t] ? 1.0 : 0.0; break;
                    case Op::Ge: for (int t = 0; t < kBlock; ++t) l[t] = l[t] >= r[t] ? 1.0 : 0.0; break;
                    case Op::Gt: for (int t = 0; t < kBlock; ++t) l[t] = l[t] > r[t] ? 1.0 : 0.0; break;
                    default: for (int t = 0; t < kBlock; ++t) l[t] = apply_binary(in.op, l[t], r[t]); break;
                }
                --sp;
                break;
            }
            case Instr::Tern: {
                double* c = &stack[(sp - 3) * kBlock];
                double* x = &stack[(sp - 2) * kBlock];
                double* y = &stack[(sp - 1) * kBlock];
                for (int t = 0; t < kBlock; ++t) c[t] = c[t] != 0 ? x[t] : y[t];
                sp -= 2;
                break;
            }
        }
    }
    std::memcpy(out, stack.data(), sizeof(double) * kBlock);
}

// The same evaluation, bit-sliced where it can be: a stack entry is a scalar constant, a 64-bit
// mask (a 0/1 value per assignment: node bits, logical operators and comparisons of 0/1 values)
// or a vector of 64 doubles (arithmetic). Logical operators and comparisons always give 0.0 or
// 1.0, so masks stand for exactly the doubles run_block would hold; arithmetic and comparisons
// that need real values expand their operands to vectors and use run_block's rules. Results are
// identical to run_block's; the usual `@logic ? rate : 0` forms never leave masks and scalars.
struct Slot {
    enum Kind { Scalar, Mask, Vec } kind;
    double c;
    uint64_t m;
    double* v;
};

uint64_t bit_pattern(uint64_t a0, int bit) {
    static const uint64_t low[6] = {0xAAAAAAAAAAAAAAAAull, 0xCCCCCCCCCCCCCCCCull, 0xF0F0F0F0F0F0F0F0ull,
                                    0xFF00FF00FF00FF00ull, 0xFFFF0000FFFF0000ull, 0xFFFFFFFF00000000ull};
    if (bit < 6) return low[bit];
    return ((a0 >> bit) & 1u) ? ~0ull : 0ull;
}

uint64_t as_mask(const Slot& s) {  // truthiness per assignment
    if (s.kind == Slot::Mask) return s.m;
    if (s.kind == Slot::Scalar) return s.c != 0 ? ~0ull : 0ull;
    uint64_t m = 0;
    for (int t = 0; t < kBlock; ++t) m |= (uint64_t)(s.v[t] != 0) << t;
    return m;
}

void as_vec(const Slot& s, double* out) {
    if (s.kind == Slot::Vec) {
        if (s.v != out) std::memcpy(out, s.v, sizeof(double) * kBlock);
    } else if (s.kind == Slot::Scalar) {
        for (int t = 0; t < kBlock; ++t) out[t] = s.c;
    } else {
        for (int t = 0; t < kBlock; ++t) out[t] = (double)((s.m >> t) & 1u);
    }
}

uint64_t compare_masks(Op op, uint64_t a, uint64_t b) {
    switch (op) {
        case Op::Eq: return ~(a ^ b);
        case Op::Ne: return a ^ b;
        case Op::Lt: return ~a & b;
        case Op::Le: return ~a | b;
        case Op::Gt: return a & ~b;
        default: return a | ~b;  // Ge
    }
}

bool is_compare(Op op) {
    return op == Op::Eq || op == Op::Ne || op == Op::Lt || op == Op::Le || op == Op::Gt || op == Op::Ge;
}

void run_block_bits(const std::vector<Instr>& prog, uint64_t a0, std::vector<double>& store, std::vector<Slot>& st,
                    double* out) {
    size_t sp = 0;
    auto vec_at = [&](size_t i) { return &store[i * kBlock]; };
    for (const Instr& in : prog) {
        switch (in.code) {
            case Instr::Const: st[sp++] = Slot{Slot::Scalar, in.c, 0, nullptr}; break;
            case Instr::Bit: st[sp++] = Slot{Slot::Mask, 0, bit_pattern(a0, in.bit), nullptr}; break;
            case Instr::Un: {
                Slot& x = st[sp - 1];
                if (in.op == Op::Plus) break;
                if (x.kind == Slot::Scalar) {
                    x.c = apply_unary(in.op, x.c);
                } else if (in.op == Op::Not) {
                    x = Slot{Slot::Mask, 0, ~as_mask(x), nullptr};
                } else {
                    double* d = vec_at(sp - 1);
                    as_vec(x, d);
                    for (int t = 0; t < kBlock; ++t) d[t] = apply_unary(in.op, d[t]);
                    x = Slot{Slot::Vec, 0, 0, d};
                }
                break;
            }
            case Instr::Bin: {
                Slot& l = st[sp - 2];
                const Slot r = st[sp - 1];
                --sp;
                if (l.kind == Slot::Scalar && r.kind == Slot::Scalar) {
                    l.c = apply_binary(in.op, l.c, r.c);
                } else if (in.op == Op::And || in.op == Op::Or || in.op == Op::Xor) {
                    const uint64_t a = as_mask(l), b = as_mask(r);
                    l = Slot{Slot::Mask, 0, in.op == Op::And ? (a & b) : in.op == Op::Or ? (a | b) : (a ^ b), nullptr};
                } else if (is_compare(in.op) && l.kind == Slot::Mask && r.kind == Slot::Mask) {
                    l = Slot{Slot::Mask, 0, compare_masks(in.op, l.m, r.m), nullptr};
                } else {
                    double* dl = vec_at(sp - 1);
                    double rv[kBlock];
                    as_vec(l, dl);
                    as_vec(r, rv);
                    if (is_compare(in.op)) {
                        uint64_t m = 0;
                        for (int t = 0; t < kBlock; ++t) m |= (uint64_t)(apply_binary(in.op, dl[t], rv[t]) != 0) << t;
                        l = Slot{Slot::Mask, 0, m, nullptr};
                    } else {
                        for (int t = 0; t < kBlock; ++t) dl[t] = apply_binary(in.op, dl[t], rv[t]);
                        l = Slot{Slot::Vec, 0, 0, dl};
                    }
                }
                break;
            }
            case Instr::Tern: {
                const uint64_t c = as_mask(st[sp - 3]);
                const Slot x = st[sp - 2], y = st[sp - 1];
                sp -= 2;
                if (c == ~0ull) {
                    st[sp - 1] = x;
                } else if (c == 0) {
                    st[sp - 1] = y;
                } else if (x.kind == Slot::Scalar && y.kind == Slot::Scalar && x.c == 1.0 && y.c == 0.0) {
                    st[sp - 1] = Slot{Slot::Mask, 0, c, nullptr};
                } else {
                    double xv[kBlock], yv[kBlock];
                    as_vec(x, xv);
                    as_vec(y, yv);
                    double* d = vec_at(sp - 1);
                    for (int t = 0; t < kBlock; ++t) d[t] = ((c >> t) & 1u) ? xv[t] : yv[t];
                    st[sp - 1] = Slot{Slot::Vec, 0, 0, d};
                }
                if (st[sp - 1].kind == Slot::Vec && st[sp - 1].v != vec_at(sp - 1)) {
                    // a branch's vector moved down the stack: keep it in its own slot's storage
                    std::memcpy(vec_at(sp - 1), st[sp - 1].v, sizeof(double) * kBlock);
                    st[sp - 1].v = vec_at(sp - 1);
                }
                break;
            }
        }
    }
    as_vec(st[0], out);
}

size_t stack_depth(const std::vector<Instr>& prog) {
    size_t sp = 0, mx = 0;
    for (const Instr& in : prog) {
        if (in.code == Instr::Const || in.code == Instr::Bit) ++sp;
        else if (in.code == Instr::Bin) --sp;
        else if (in.code == Instr::Tern) sp -= 2;
        mx = std::max(mx, sp);
    }
    return mx;
}

}  // namespace

uint64_t quantize_rate(double r, int frac_bits) {
    double q = std::nearbyint(std::ldexp(r, frac_bits));
    if (!(q < 18446744073709551616.0)) throw Error("rate too large for fixed point");
    uint64_t v = (uint64_t)q;
    if (v == 0 && r > 0) v = 1;  // a positive rate stays able to fire
    return v;
}

static int frac_bits_for(double sum_max) {
    // fixed-point scale: the sum of every node's largest rate stays below 2^61
    int fb = 40;
    if (sum_max > 0) fb = std::min(40, (int)std::floor(61.0 - std::log2(sum_max)));
    if (fb < 8) throw Error("rates too large for the fixed-point representation");
    return fb;
}

// Binary form (one up rate, one down rate, a bit per assignment saying whether the rate is
// non-zero) when every non-zero up value is equal and every non-zero down value is equal,
// palette form otherwise. `tab` holds the node's rate per assignment (self bit k).
static void classify_node(CompiledNode& cn, const std::vector<double>& tab, int fb, const std::string& name) {
    const int k = (int)cn.regs.size();
    const uint64_t half = 1ull << k, total = half << 1;
    // the binary form needs at most one distinct non-zero value per half
    double upv = 0, dnv = 0;
    bool binary = true;
    for (uint64_t a = 0; a < total && binary; ++a) {
        if (tab[a] == 0) continue;
        double& v = a < half ? upv : dnv;
        if (v == 0) v = tab[a];
        else if (v != tab[a]) binary = false;
    }
    cn.bits.clear();
    cn.pidx.clear();
    cn.palette.clear();
    cn.palette_real.clear();
    if (binary) {
        cn.kind = NODE_BINARY;
        cn.up_real = upv;
        cn.down_real = dnv;
        cn.up = quantize_rate(cn.up_real, fb);
        cn.down = quantize_rate(cn.down_real, fb);
        cn.bits.assign((total + 31) / 32, 0u);
        for (uint64_t a = 0; a < total; ++a)
            if (tab[a] != 0) cn.bits[a >> 5] |= 1u << (a & 31);
    } else {
        if (k > kMaxPaletteRegs)
            throw Error("node " + name + " has a multi-valued rate over " + std::to_string(k) + " nodes (limit " +
                        std::to_string(kMaxPaletteRegs) + ")");
        std::set<double> all(tab.begin(), tab.end());
        if (all.size() > 256) throw Error("node " + name + " has more than 256 distinct rates");
        cn.kind = NODE_PALETTE;
        cn.up = cn.down = 0;
        cn.up_real = cn.down_real = 0;
        cn.palette_real.assign(all.begin(), all.end());
        for (double r : cn.palette_real) cn.palette.push_back(quantize_rate(r, fb));
        cn.pidx.resize(total);
        for (uint64_t a = 0; a < total; ++a)
            cn.pidx[a] = (uint8_t)(std::lower_bound(cn.palette_real.begin(), cn.palette_real.end(), tab[a]) -
                                   cn.palette_real.begin());
    }
}

// The node's rate per assignment, in double, rebuilt from its compiled form.
static std::vector<double> node_table(const CompiledNode& cn) {
    const int k = (int)cn.regs.size();
    const uint64_t half = 1ull << k, total = half << 1;
    std::vector<double> tab(total, 0.0);
    for (uint64_t a = 0; a < total; ++a) {
        if (cn.kind == NODE_BINARY) {
            if ((cn.bits[a >> 5] >> (a & 31)) & 1u) tab[a] = a < half ? cn.up_real : cn.down_real;
        } else {
            tab[a] = cn.palette_real[cn.pidx[a]];
        }
    }
    return tab;
}

static double node_max_rate(const CompiledNode& cn) {
    if (cn.kind == NODE_PALETTE) return cn.palette_real.empty() ? 0.0 : cn.palette_real.back();
    const int k = (int)cn.regs.size();
    const uint64_t half = 1ull << k, total = half << 1;
    bool any_up = false, any_down = false;
    for (uint64_t a = 0; a < total; ++a)
        if ((cn.bits[a >> 5] >> (a & 31)) & 1u) (a < half ? any_up : any_down) = true;
    return std::max(any_up ? cn.up_real : 0.0, any_down ? cn.down_real : 0.0);
}

CompiledModel mutate_model(const CompiledModel& src, const int* nodes, const int* values, int count) {
    CompiledModel cm = src;
    std::vector<int> value(cm.n, -1);
    for (int j = 0; j < count; ++j) {
        if (nodes[j] < 0 || nodes[j] >= cm.n) throw Error("mutant node index out of range");
        if (values[j] != 0 && values[j] != 1) throw Error("mutant value must be 0 (OFF) or 1 (ON)");
        value[nodes[j]] = values[j];
    }
    std::vector<std::vector<double>> tabs(cm.n);
    double sum_max = 0;
    for (int i = 0; i < cm.n; ++i) {
        CompiledNode& cn = cm.nodes[i];
        if (value[i] < 0) {
            sum_max += node_max_rate(cn);
            continue;
        }
        // the node leaves `value` at rate 0: assignments whose self bit equals the value
        tabs[i] = node_table(cn);
        const int k = (int)cn.regs.size();
        const uint64_t half = 1ull << k, total = half << 1;
        for (uint64_t a = value[i] ? half : 0; a < (value[i] ? total : half); ++a) tabs[i][a] = 0.0;
        double mx = 0;
        for (double r : tabs[i]) mx = std::max(mx, r);
        sum_max += mx;
        cm.istate[i] = value[i];
        cm.istate_thr[i] = value[i] ? 16777216u : 0u;
    }
    cm.frac_bits = frac_bits_for(sum_max);
    for (int i = 0; i < cm.n; ++i) {
        CompiledNode& cn = cm.nodes[i];
        if (value[i] >= 0) {
            classify_node(cn, tabs[i], cm.frac_bits, "#" + std::to_string(i));
        } else if (cn.kind == NODE_BINARY) {
            cn.up = quantize_rate(cn.up_real, cm.frac_bits);
            cn.down = quantize_rate(cn.down_real, cm.frac_bits);
        } else {
            for (size_t q = 0; q < cn.palette.size(); ++q) cn.palette[q] = quantize_rate(cn.palette_real[q], cm.frac_bits);
        }
    }
    return cm;
}

CompiledModel rescale_model(const CompiledModel& src, const double* up_scale, const double* down_scale) {
    CompiledModel cm = src;
    double sum_max = 0;
    for (int i = 0; i < cm.n; ++i) {
        CompiledNode& cn = cm.nodes[i];
        if (cn.kind != NODE_BINARY) throw Error("rate scaling of multi-valued rates is not supported");
        const double su = up_scale ? up_scale[i] : 1.0, sd = down_scale ? down_scale[i] : 1.0;
        if (!(su >= 0) || !(sd >= 0) || std::isinf(su) || std::isinf(sd)) throw Error("invalid rate scale");
        cn.up_real *= su;
        cn.down_real *= sd;
        sum_max += std::max(cn.up_real, cn.down_real);
    }
    cm.frac_bits = frac_bits_for(sum_max);
    for (auto& cn : cm.nodes) {
        cn.up = quantize_rate(cn.up_real, cm.frac_bits);
        cn.down = quantize_rate(cn.down_real, cm.frac_bits);
    }
    return cm;
}

CompiledModel compile_arrays(int n, const int32_t* reg_off, const int32_t* regs, const uint32_t* logic,
                             int64_t logic_words, const int64_t* logic_off, const double* rate_up,
                             const double* rate_down, const double* istate, const uint8_t* is_output,
                             const RunConstants& rc) {
    if (n < 1) throw Error("model has no nodes");
    if (n > kMaxNodes) throw Error("model has more than 65535 nodes");
    if (!reg_off || !logic || !logic_off || !rate_up || !rate_down || !istate)
        throw Error("null model array");
    if (reg_off[0] != 0) throw Error("reg_off[0] must be 0");
    for (int i = 0; i < n; ++i)
        if (reg_off[i + 1] < reg_off[i]) throw Error("reg_off must not decrease");
    if (reg_off[n] > 0 && !regs) throw Error("null regulator array");
    CompiledModel cm;
    cm.n = n;
    cm.words = (n + 31) / 32;
    cm.nodes.resize(n);
    cm.out_pos.assign(n, -1);
    for (int i = 0; i < n; ++i)
        if (!is_output || is_output[i]) {
            cm.out_pos[i] = (int)cm.out_nodes.size();
            cm.out_nodes.push_back(i);
        }
    cm.n_out = (int)cm.out_nodes.size();
    double sum_max = 0;
    for (int i = 0; i < n; ++i) {
        const int k = reg_off[i + 1] - reg_off[i];
        const std::string name = "#" + std::to_string(i);
        if (k > kMaxBinaryRegs)
            throw Error("node " + name + " reads " + std::to_string(k) + " nodes (limit " +
                        std::to_string(kMaxBinaryRegs) + ")");
        const double up = rate_up[i], down = rate_down[i];
        if (!(up >= 0) || !(down >= 0) || std::isinf(up) || std::isinf(down))
            throw Error("node " + name + " has a negative or non-finite rate");
        // regulators in ascending order, and where each one sits in the caller's order
        std::vector<std::pair<int, int>> order;
        for (int j = 0; j < k; ++j) {
            const int r = regs[reg_off[i] + j];
            if (r < 0 || r >= n || r == i) throw Error("node " + name + " has a regulator out of range or itself");
            order.push_back({r, j});
        }
        std::sort(order.begin(), order.end());
        for (int j = 1; j < k; ++j)
            if (order[j].first == order[j - 1].first) throw Error("node " + name + " lists a regulator twice");
        CompiledNode& cn = cm.nodes[i];
        for (auto& o : order) cn.regs.push_back(o.first);
        cm.max_k = std::max(cm.max_k, k);
        const uint64_t half = 1ull << k, total = half << 1;
        const int64_t words = (int64_t)((half + 31) / 32);
        if (logic_off[i] < 0 || logic_off[i] > logic_words - words)
            throw Error("node " + name + ": its truth table lies outside the logic array");
        cn.kind = NODE_BINARY;
        cn.up_real = up;
        cn.down_real = down;
        cn.bits.assign((total + 31) / 32, 0u);
        const uint32_t* tab = logic + logic_off[i];
        bool any_up = false, any_down = false;
        for (uint64_t a = 0; a < half; ++a) {
            uint64_t idx = 0;  // the assignment's index in the caller's regulator order
            for (int j = 0; j < k; ++j) idx |= ((a >> j) & 1ull) << order[j].second;
            const bool on = (tab[idx >> 5] >> (idx & 31)) & 1u;
            if (on && up > 0) {
                cn.bits[a >> 5] |= 1u << (a & 31);
                any_up = true;
            }
            if (!on && down > 0) {
                const uint64_t b = a + half;
                cn.bits[b >> 5] |= 1u << (b & 31);
                any_down = true;
            }
        }
        sum_max += std::max(any_up ? up : 0.0, any_down ? down : 0.0);
    }
    cm.frac_bits = frac_bits_for(sum_max);
    for (auto& cn : cm.nodes) {
        cn.up = quantize_rate(cn.up_real, cm.frac_bits);
        cn.down = quantize_rate(cn.down_real, cm.frac_bits);
    }
    cm.deps.assign(n, {});
    for (int i = 0; i < n; ++i) {
        cm.deps[i].push_back(i);
        for (int r : cm.nodes[i].regs) cm.deps[r].push_back(i);
    }
    for (auto& d : cm.deps) {
        std::sort(d.begin(), d.end());
        d.erase(std::unique(d.begin(), d.end()), d.end());
    }
    cm.istate.resize(n);
    cm.istate_thr.resize(n);
    for (int i = 0; i < n; ++i) {
        const double p = istate[i];
        if (!(p >= 0 && p <= 1)) throw Error("istate of node #" + std::to_string(i) + " is outside [0, 1]");
        cm.istate[i] = p;
        cm.istate_thr[i] = (uint32_t)std::floor(p * 16777216.0);
    }
    cm.discrete = rc.discrete;
    cm.max_time = rc.max_time;
    cm.tick = rc.tick;
    cm.sample_count = rc.sample_count;
    cm.seed = rc.seed;
    if (!(cm.max_time > 0) || !(cm.tick > 0)) throw Error("max_time and time_tick must be positive");
    cm.windows = (int)std::ceil((float)cm.max_time / (float)cm.tick);
    if (cm.windows < 1) cm.windows = 1;
    return cm;
}


CompiledModel compile_model(const Model& m) {
    CompiledModel cm;
    cm.n = (int)m.nodes.size();
    if (cm.n == 0) throw Error("model has no nodes");
    if (cm.n > kMaxNodes) throw Error("model has more than 65535 nodes");
    cm.words = (cm.n + 31) / 32;
    cm.nodes.resize(cm.n);
    cm.out_pos.assign(cm.n, -1);
    for (int i = 0; i < cm.n; ++i) {
        if (!m.is_internal(i)) {
            cm.out_pos[i] = (int)cm.out_nodes.size();
            cm.out_nodes.push_back(i);
        }
    }
    cm.n_out = (int)cm.out_nodes.size();

    // Tabulate every node's rate over (self, regulators) in double, nodes spread over host threads
    // (a node with 20 regulators alone is 2^21 entries); each node's result depends on it alone.
    std::vector<std::vector<double>> tabs(cm.n);
    std::vector<double> node_max(cm.n, 0.0);
    struct Scratch {
        std::vector<int> sup, inputs;
        std::vector<Instr> pu, pd;
        std::vector<double> stack;
        std::vector<Slot> slots;
    };
    auto tabulate = [&](int i, Scratch& sc) {
        const Node& nd = m.nodes[i];
        const Expr* up = nd.attr("rate_up");
        const Expr* down = nd.attr("rate_down");
        if (!up || !down) throw Error("Node " + nd.name + " lacks rate_up or rate_down");
        sc.sup.clear();
        collect_support(*up, m, i, sc.sup);
        collect_support(*down, m, i, sc.sup);
        std::sort(sc.sup.begin(), sc.sup.end());
        sc.sup.erase(std::unique(sc.sup.begin(), sc.sup.end()), sc.sup.end());
        CompiledNode& cn = cm.nodes[i];
        for (int s : sc.sup)
            if (s != i) cn.regs.push_back(s);
        const int k = (int)cn.regs.size();
        if (k > kMaxBinaryRegs)
            throw Error("node " + nd.name + " reads " + std::to_string(k) + " nodes (limit " +
                        std::to_string(kMaxBinaryRegs) + ")");
        sc.inputs.assign(cn.regs.begin(), cn.regs.end());
        sc.inputs.push_back(i);  // input bit k is the node itself
        sc.pu.clear();
        sc.pd.clear();
        flatten(*up, m, i, sc.inputs, sc.pu, 0);
        flatten(*down, m, i, sc.inputs, sc.pd, 0);
        const size_t depth = std::max(stack_depth(sc.pu), stack_depth(sc.pd)) + 1;
        sc.stack.assign(kBlock * depth, 0.0);
        sc.slots.assign(depth, Slot{});
        const uint64_t half = 1ull << k, total = half << 1;
        std::vector<double>& tab = tabs[i];
        tab.assign(std::max<uint64_t>(total, kBlock), 0.0);
        double buf[kBlock];
        // assignments with the self bit (bit k) clear read rate_up, set read rate_down: rate_up
        // runs over the lower half only, rate_down over the upper half only (a block never
        // straddles the halves when half >= kBlock)
        for (uint64_t a0 = 0; a0 < total; a0 += kBlock) {
            const uint64_t n_here = std::min<uint64_t>(kBlock, total - a0);
            const bool any_up = a0 < half, any_down = a0 + n_here > half;
            if (any_up) {
                run_block_bits(sc.pu, a0, sc.stack, sc.slots, buf);
                for (uint64_t t = 0; t < n_here; ++t)
                    if (!(((a0 + t) >> k) & 1u)) tab[a0 + t] = buf[t];
            }
            if (any_down) {
                run_block_bits(sc.pd, a0, sc.stack, sc.slots, buf);
                for (uint64_t t = 0; t < n_here; ++t)
                    if (((a0 + t) >> k) & 1u) tab[a0 + t] = buf[t];
            }
        }
        tab.resize(total);
        double mx = 0;
        for (double r : tab) {
            if (!(r >= 0) || std::isinf(r))
                throw Error("node " + nd.name + " has a negative or non-finite rate");
            mx = std::max(mx, r);
        }
        node_max[i] = mx;
    };
    parallel_items<Scratch>(cm.n, 256, [&](int i, Scratch& sc) { tabulate(i, sc); });
    double sum_max = 0;
    for (int i = 0; i < cm.n; ++i) {
        sum_max += node_max[i];  // node order, as one thread would add them
        cm.max_k = std::max(cm.max_k, (int)cm.nodes[i].regs.size());
    }

    const int fb = frac_bits_for(sum_max);
    cm.frac_bits = fb;

    parallel_items<int>(cm.n, 256, [&](int i, int&) { classify_node(cm.nodes[i], tabs[i], fb, m.nodes[i].name); });

    cm.deps.assign(cm.n, {});
    for (int i = 0; i < cm.n; ++i) {
        cm.deps[i].push_back(i);
        for (int r : cm.nodes[i].regs) cm.deps[r].push_back(i);
    }
    for (auto& d : cm.deps) {
        std::sort(d.begin(), d.end());
        d.erase(std::unique(d.begin(), d.end()), d.end());
    }

    cm.istate.resize(cm.n);
    cm.istate_thr.resize(cm.n);
    for (int i = 0; i < cm.n; ++i) {
        double p = m.nodes[i].istate;
        if (!(p >= 0 && p <= 1)) throw Error("istate of node " + m.nodes[i].name + " is outside [0, 1]");
        cm.istate[i] = p;
        cm.istate_thr[i] = (uint32_t)std::floor(p * 16777216.0);
    }

    // run constants (main.cpp:128-132)
    cm.discrete = m.constant("discrete_time") != 0;
    cm.max_time = m.constant("max_time");
    cm.tick = m.constant("time_tick");
    double sc = m.constant("sample_count");
    cm.sample_count = sc > 0 ? (uint64_t)sc : 0;
    double seed = m.constant("seed_pseudorandom");
    cm.seed = seed > 0 ? (uint64_t)seed : 0;
    if (!(cm.max_time > 0) || !(cm.tick > 0)) throw Error("max_time and time_tick must be positive");
    // window count as the reference computes it, in float (window_average_small.cpp:26)
    cm.windows = (int)std::ceil((float)cm.max_time / (float)cm.tick);
    if (cm.windows < 1) cm.windows = 1;
    return cm;
}

}  // namespace mbg
