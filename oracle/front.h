// Front end of the host FP64 oracle: TEST INFRASTRUCTURE ONLY, written apart from the product so
// that a defect of the product's parser, tables or random streams cannot appear on both sides of a
// parity test. Everything here restates the reference or a published algorithm:
//   tokens                 src/parser/scanner.ll:51-94 (keywords case-insensitive, `//` comments,
//                          TRUE/FALSE as 1/0, `$var`, `@alias`; `[`, `]`, `,` added for the istate
//                          form the grammar declares)
//   grammar, precedence    src/parser/parser.yy:74-158, 126-134 (?: lowest and right-associative,
//                          then XOR, OR, AND, == !=, < <= > >=, + -, * /, unary - + NOT)
//   declarations           src/parser/driver.cpp:7-99 (constant defaults, node registration with
//                          rate_up and rate_down required, `istate` attribute, the bracket istate
//                          form), src/parser/parse_types.cpp:3-23 (istate 0.5, first attribute of
//                          a name wins, is_internal)
//   expression values      evaluated in double (the reference evaluates in float; the product
//                          documents double)
//   Philox4x32-10          Salmon, Moraes, Dror and Shaw, "Parallel Random Numbers: As Easy as 1,
//                          2, 3", SC'11 (round function, multipliers and Weyl key increments)
//   stream layout and      the simulator's documented stream: key = seed; step s of trajectory j
//   fixed-point rules      has counter (s, j) and words (dt, pick high, pick low); initial-state
//                          block b has counter (b, 0xFFFFFFFF, j); dt uniform ((u >> 8) + 1) / 2^24;
//                          pick target floor(U64 * total / 2^64); rates rounded to F fraction bits,
//                          F = min(40, floor(61 - log2 sum of every node's largest rate)), a positive
//                          rate never below one unit
#pragma once

#include <cctype>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace orc {

struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------------------------
// Random streams.

struct W4 {
    uint32_t x, y, z, w;
};

inline W4 philox10(W4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const W4 n = {(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

inline W4 step_draws(uint64_t seed, uint64_t traj, uint64_t step) {
    return philox10({(uint32_t)step, (uint32_t)(step >> 32), (uint32_t)traj, (uint32_t)(traj >> 32)}, (uint32_t)seed,
                    (uint32_t)(seed >> 32));
}

inline W4 init_draws(uint64_t seed, uint64_t traj, uint32_t block) {
    return philox10({block, 0xFFFFFFFFu, (uint32_t)traj, (uint32_t)(traj >> 32)}, (uint32_t)seed,
                    (uint32_t)(seed >> 32));
}

inline double unit_open0(uint32_t u) { return (double)((u >> 8) + 1u) / 16777216.0; }

inline uint64_t pick_target(uint32_t hi, uint32_t lo, uint64_t total) {
    const unsigned __int128 u = ((unsigned __int128)(((uint64_t)hi << 32) | lo)) * total;
    return (uint64_t)(u >> 64);
}

inline uint64_t quantize(double r, int bits) {
    if (r < 0) throw Error("negative rate");
    const double q = std::nearbyint(std::ldexp(r, bits));
    if (!(q < 18446744073709551616.0)) throw Error("rate too large for fixed point");
    uint64_t v = (uint64_t)q;
    if (v == 0 && r > 0) v = 1;
    return v;
}

inline int frac_bits_for(double sum_max) {
    int fb = 40;
    if (sum_max > 0) fb = std::min(40, (int)std::floor(61.0 - std::log2(sum_max)));
    if (fb < 8) throw Error("rates too large for the fixed-point representation");
    return fb;
}

enum Status : uint8_t { CONTINUE = 0, FINISHED = 1, FIXED_POINT = 2, STEP_LIMIT = 3, FAILED = 4 };

// ---------------------------------------------------------------------------------------------
// Expressions.

enum class Op { Add, Sub, Mul, Div, And, Or, Xor, Not, Neg, Pos, Eq, Ne, Lt, Le, Gt, Ge };

struct Expr {
    enum Kind { Num, Node, Var, Alias, Unary, Binary, Ternary } kind = Num;
    double value = 0;
    std::string name;
    Op op = Op::Add;
    std::unique_ptr<Expr> a, b, c;
};
using ExprP = std::unique_ptr<Expr>;

struct NodeDef {
    std::string name;
    std::vector<std::pair<std::string, ExprP>> attrs;  // in declaration order: the first of a name wins
    double istate = 0.5;
    const Expr* attr(const std::string& n) const {
        for (const auto& a : attrs)
            if (a.first == n) return a.second.get();
        return nullptr;
    }
};

struct ModelDef {
    std::vector<NodeDef> nodes;
    std::unordered_map<std::string, int> index;
    std::map<std::string, double> vars;
    std::map<std::string, double> consts = {
        {"discrete_time", 0}, {"sample_count", 1000000}, {"max_time", 10}, {"time_tick", 0.1}, {"seed_pseudorandom", 0}};
    double constant(const std::string& n) const {
        auto it = consts.find(n);
        return it == consts.end() ? 0.0 : it->second;
    }
};

inline double apply(Op op, double l, double r) {
    switch (op) {
        case Op::Add: return l + r;
        case Op::Sub: return l - r;
        case Op::Mul: return l * r;
        case Op::Div: return l / r;
        case Op::And: return (l != 0 && r != 0) ? 1 : 0;
        case Op::Or: return (l != 0 || r != 0) ? 1 : 0;
        case Op::Xor: return ((l != 0) != (r != 0)) ? 1 : 0;
        case Op::Eq: return l == r;
        case Op::Ne: return l != r;
        case Op::Lt: return l < r;
        case Op::Le: return l <= r;
        case Op::Gt: return l > r;
        case Op::Ge: return l >= r;
        case Op::Neg: return -r;
        case Op::Pos: return r;
        case Op::Not: return r == 0 ? 1 : 0;
    }
    return 0;
}

// Value of a constant expression (variables allowed, nodes and aliases not).
inline double eval_const(const Expr& e, const ModelDef& m) {
    switch (e.kind) {
        case Expr::Num: return e.value;
        case Expr::Var: {
            auto it = m.vars.find(e.name);
            if (it == m.vars.end()) throw Error("unknown variable " + e.name);
            return it->second;
        }
        case Expr::Node: throw Error("node " + e.name + " in an expression that must be constant");
        case Expr::Alias: throw Error("alias " + e.name + " in an expression that must be constant");
        case Expr::Unary: return apply(e.op, 0, eval_const(*e.a, m));
        case Expr::Binary: return apply(e.op, eval_const(*e.a, m), eval_const(*e.b, m));
        case Expr::Ternary: return eval_const(*e.a, m) != 0 ? eval_const(*e.b, m) : eval_const(*e.c, m);
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Lexer and parser.

struct Tok {
    enum Kind { End, Num, Id, Var, Alias, Sym } kind = End;
    std::string text;  // identifier, symbol
    double value = 0;
    int line = 1;
};

class Parser {
public:
    Parser(const std::string& src, const std::string& file) : s_(src), file_(file) { next(); }

    void bnd(ModelDef& m) {
        while (t_.kind != Tok::End) {
            std::string kw = expect_id();
            for (char& ch : kw) ch = (char)std::tolower((unsigned char)ch);
            if (kw != "node") fail("expected 'node' keyword");
            NodeDef nd;
            nd.name = expect_id();
            expect("{");
            do {
                std::string an = expect_id();
                expect("=");
                ExprP e = expr();
                expect(";");
                nd.attrs.emplace_back(std::move(an), std::move(e));
            } while (!is("}"));
            expect("}");
            if (m.index.count(nd.name)) fail("Node " + nd.name + " already exists");
            if (!nd.attr("rate_up")) fail("Node " + nd.name + " does not have rate_up attribute");
            if (!nd.attr("rate_down")) fail("Node " + nd.name + " does not have rate_down attribute");
            m.index.emplace(nd.name, (int)m.nodes.size());
            m.nodes.push_back(std::move(nd));
        }
    }

    void cfg(ModelDef& m) {
        while (t_.kind != Tok::End) {
            if (t_.kind == Tok::Var) {  // $var = exp;
                std::string v = t_.text;
                next();
                expect("=");
                ExprP e = expr();
                expect(";");
                m.vars[v] = eval_const(*e, m);
            } else if (is("[")) {  // [node].istate = p [a], q [b];
                next();
                const std::string node = expect_id();
                expect("]");
                expect(".");
                if (expect_id() != "istate") fail("expected 'istate' keyword");
                expect("=");
                ExprP e1 = expr();
                const int a = bracket_number();
                expect(",");
                ExprP e2 = expr();
                const int b = bracket_number();
                expect(";");
                if (!((a == 0 && b == 1) || (a == 1 && b == 0))) fail("numbers in [] must be 0 and 1");
                const double p = eval_const(*e1, m), q = eval_const(*e2, m);
                node_of(m, node).istate = a == 1 ? p / (p + q) : q / (p + q);
            } else {
                const std::string name = expect_id();
                if (is(".")) {  // node.attr = exp;
                    next();
                    std::string attr = expect_id();
                    expect("=");
                    ExprP e = expr();
                    expect(";");
                    NodeDef& nd = node_of(m, name);
                    if (attr == "istate") nd.istate = eval_const(*e, m);
                    else nd.attrs.emplace_back(std::move(attr), std::move(e));
                } else {  // constant = exp;
                    expect("=");
                    ExprP e = expr();
                    expect(";");
                    m.consts[name] = eval_const(*e, m);
                }
            }
        }
    }

private:
    const std::string& s_;
    std::string file_;
    size_t p_ = 0;
    int line_ = 1;
    Tok t_;

    [[noreturn]] void fail(const std::string& msg) const {
        throw Error(file_ + ":" + std::to_string(t_.line) + ": " + msg);
    }

    void next() {
        for (;;) {  // blanks, newlines, // comments
            while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\r' || s_[p_] == '\n')) {
                if (s_[p_] == '\n') ++line_;
                ++p_;
            }
            if (p_ + 1 < s_.size() && s_[p_] == '/' && s_[p_ + 1] == '/') {
                while (p_ < s_.size() && s_[p_] != '\n') ++p_;
                continue;
            }
            break;
        }
        t_ = Tok();
        t_.line = line_;
        if (p_ >= s_.size()) return;
        const char c = s_[p_];
        auto ident_at = [&](size_t q) {
            size_t e = q;
            while (e < s_.size() && (std::isalnum((unsigned char)s_[e]) || s_[e] == '_')) ++e;
            return e;
        };
        if (std::isdigit((unsigned char)c) || (c == '.' && p_ + 1 < s_.size() && std::isdigit((unsigned char)s_[p_ + 1]))) {
            size_t e = p_;
            while (e < s_.size() && std::isdigit((unsigned char)s_[e])) ++e;
            if (e < s_.size() && s_[e] == '.') {
                ++e;
                while (e < s_.size() && std::isdigit((unsigned char)s_[e])) ++e;
            }
            if (e < s_.size() && (s_[e] == 'e' || s_[e] == 'E')) {
                size_t f = e + 1;
                if (f < s_.size() && (s_[f] == '+' || s_[f] == '-')) ++f;
                if (f < s_.size() && std::isdigit((unsigned char)s_[f])) {
                    while (f < s_.size() && std::isdigit((unsigned char)s_[f])) ++f;
                    e = f;
                }
            }
            t_.kind = Tok::Num;
            t_.value = std::strtod(s_.substr(p_, e - p_).c_str(), nullptr);
            p_ = e;
            return;
        }
        if (std::isalpha((unsigned char)c)) {
            const size_t e = ident_at(p_);
            std::string w = s_.substr(p_, e - p_);
            p_ = e;
            std::string u = w;
            for (char& ch : u) ch = (char)std::toupper((unsigned char)ch);
            if (u == "TRUE" || u == "FALSE") {
                t_.kind = Tok::Num;
                t_.value = u == "TRUE" ? 1 : 0;
            } else if (u == "AND" || u == "OR" || u == "XOR" || u == "NOT") {
                t_.kind = Tok::Sym;
                t_.text = u == "AND" ? "&" : u == "OR" ? "|" : u == "XOR" ? "^" : "!";
            } else {
                t_.kind = Tok::Id;
                t_.text = w;
            }
            return;
        }
        if ((c == '$' || c == '@') && p_ + 1 < s_.size() && std::isalpha((unsigned char)s_[p_ + 1])) {
            const size_t e = ident_at(p_ + 1);
            t_.kind = c == '$' ? Tok::Var : Tok::Alias;
            t_.text = s_.substr(p_, e - p_);
            p_ = e;
            return;
        }
        static const char* two[] = {"&&", "||", "==", "!=", "<=", ">="};
        for (const char* w : two)
            if (s_.compare(p_, 2, w) == 0) {
                t_.kind = Tok::Sym;
                t_.text = std::string(w) == "&&" ? "&" : std::string(w) == "||" ? "|" : w;
                p_ += 2;
                return;
            }
        if (std::string("-+*/()=?:&|^!<>{}.;[],").find(c) != std::string::npos) {
            t_.kind = Tok::Sym;
            t_.text = std::string(1, c);
            ++p_;
            return;
        }
        fail(std::string("invalid character: ") + c);
    }

    bool is(const char* sym) const { return t_.kind == Tok::Sym && t_.text == sym; }
    void expect(const char* sym) {
        if (!is(sym)) fail(std::string("expected '") + sym + "'");
        next();
    }
    std::string expect_id() {
        if (t_.kind != Tok::Id) fail("expected an identifier");
        std::string s = t_.text;
        next();
        return s;
    }
    int bracket_number() {
        expect("[");
        if (t_.kind != Tok::Num) fail("expected a number");
        const int v = (int)t_.value;
        next();
        expect("]");
        return v;
    }
    static NodeDef& node_of(ModelDef& m, const std::string& name) {
        auto it = m.index.find(name);
        if (it == m.index.end()) throw Error("Unknown node " + name);
        return m.nodes[it->second];
    }

    static ExprP make(Expr::Kind k) {
        ExprP e(new Expr());
        e->kind = k;
        return e;
    }

    ExprP expr() {  // ?: binds loosest and groups to the right
        ExprP c = binary(0);
        if (!is("?")) return c;
        next();
        ExprP t = expr();
        expect(":");
        ExprP f = expr();
        ExprP e = make(Expr::Ternary);
        e->a = std::move(c);
        e->b = std::move(t);
        e->c = std::move(f);
        return e;
    }

    // level 0: XOR, 1: OR, 2: AND, 3: == !=, 4: < <= > >=, 5: + -, 6: * /
    bool op_at(int level, Op& op) const {
        if (t_.kind != Tok::Sym) return false;
        const std::string& x = t_.text;
        switch (level) {
            case 0: if (x == "^") { op = Op::Xor; return true; } return false;
            case 1: if (x == "|") { op = Op::Or; return true; } return false;
            case 2: if (x == "&") { op = Op::And; return true; } return false;
            case 3:
                if (x == "==") { op = Op::Eq; return true; }
                if (x == "!=") { op = Op::Ne; return true; }
                return false;
            case 4:
                if (x == "<") { op = Op::Lt; return true; }
                if (x == "<=") { op = Op::Le; return true; }
                if (x == ">") { op = Op::Gt; return true; }
                if (x == ">=") { op = Op::Ge; return true; }
                return false;
            case 5:
                if (x == "+") { op = Op::Add; return true; }
                if (x == "-") { op = Op::Sub; return true; }
                return false;
            default:
                if (x == "*") { op = Op::Mul; return true; }
                if (x == "/") { op = Op::Div; return true; }
                return false;
        }
    }

    ExprP binary(int level) {
        if (level > 6) return unary();
        ExprP l = binary(level + 1);
        Op op;
        while (op_at(level, op)) {
            next();
            ExprP r = binary(level + 1);
            ExprP e = make(Expr::Binary);
            e->op = op;
            e->a = std::move(l);
            e->b = std::move(r);
            l = std::move(e);
        }
        return l;
    }

    ExprP unary() {
        if (is("-") || is("+") || is("!")) {
            const Op op = is("-") ? Op::Neg : is("+") ? Op::Pos : Op::Not;
            next();
            ExprP e = make(Expr::Unary);
            e->op = op;
            e->a = unary();
            return e;
        }
        return primary();
    }

    ExprP primary() {
        if (is("(")) {
            next();
            ExprP e = expr();
            expect(")");
            return e;
        }
        ExprP e;
        switch (t_.kind) {
            case Tok::Num: e = make(Expr::Num); e->value = t_.value; break;
            case Tok::Id: e = make(Expr::Node); e->name = t_.text; break;
            case Tok::Var: e = make(Expr::Var); e->name = t_.text; break;
            case Tok::Alias: e = make(Expr::Alias); e->name = t_.text; break;
            default: fail("unexpected token in expression");
        }
        next();
        return e;
    }
};

inline void parse_model(ModelDef& m, const std::string& bnd, const std::string& cfg) {
    Parser(bnd, "model.bnd").bnd(m);
    Parser(cfg, "model.cfg").cfg(m);
}

inline bool is_internal(const ModelDef& m, int i) {
    const Expr* e = m.nodes[i].attr("is_internal");
    return e && eval_const(*e, m) != 0;
}

}  // namespace orc
