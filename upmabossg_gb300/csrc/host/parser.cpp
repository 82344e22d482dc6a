// Hand-written lexer and precedence-climbing parser for the .bnd / .cfg grammar.
//
// Token set follows src/parser/scanner.ll:51-94 (keywords AND/OR/XOR/NOT/TRUE/FALSE are case
// insensitive and win over identifiers of the same length; `//` comments; `$var`, `@alias`).
// Productions follow src/parser/parser.yy:74-158 and the operator precedence of
// parser.yy:126-134, lowest first: `?:` (right), XOR, OR, AND, `== !=`, `< <= > >=`, `+ -`,
// `* /`, unary `- + !`.
#include <cctype>
#include <cerrno>
#include <climits>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "model.hpp"

namespace mbg {

namespace {

enum class Tok {
    Eof, Ident, Var, Alias, Number, Float,
    Minus, Plus, Star, Slash, LParen, RParen, Assign, Question, Colon,
    And, Or, Xor, Not, Eq, Ne, Lt, Le, Gt, Ge, LBrace, RBrace, Dot, Semi,
    LBracket, RBracket, Comma,
};

struct Token {
    Tok t = Tok::Eof;
    std::string text;
    double num = 0;
    int line = 1, col = 1;
};

// ASCII character classes (the grammar is ASCII; no locale lookups).
inline bool is_alpha(char c) { return (unsigned)((c | 0x20) - 'a') < 26u; }
inline bool is_digit(char c) { return (unsigned)(c - '0') < 10u; }
inline bool is_ident(char c) { return is_alpha(c) || is_digit(c) || c == '_'; }

bool ieq(const std::string& a, const char* b) {
    size_t n = 0;
    for (; b[n]; ++n) {
        if (n >= a.size() || std::tolower((unsigned char)a[n]) != std::tolower((unsigned char)b[n])) return false;
    }
    return n == a.size();
}

class Lexer {
public:
    Lexer(const std::string& src, const std::string& fname) : s_(src), f_(fname) {
        if (s_.size() >= 3 && (unsigned char)s_[0] == 0xEF && (unsigned char)s_[1] == 0xBB &&
            (unsigned char)s_[2] == 0xBF)
            p_ = 3;
    }

    [[noreturn]] void fail(int line, int col, const std::string& msg) const {
        throw Error(f_ + ":" + std::to_string(line) + ":" + std::to_string(col) + ": " + msg);
    }

    Token next() {
        skip();
        Token tk;
        tk.line = line_;
        tk.col = col_;
        if (p_ >= s_.size()) return tk;
        char c = s_[p_];
        if (is_alpha(c)) {
            size_t b = p_;
            while (p_ < s_.size() && is_ident(s_[p_])) ++p_;  // no newline inside a word
            col_ += (int)(p_ - b);
            tk.text.assign(s_, b, p_ - b);
            tk.t = Tok::Ident;
            if (tk.text.size() <= 5) {  // keywords: AND OR XOR NOT TRUE FALSE, any case
                if (ieq(tk.text, "AND")) tk.t = Tok::And;
                else if (ieq(tk.text, "OR")) tk.t = Tok::Or;
                else if (ieq(tk.text, "XOR")) tk.t = Tok::Xor;
                else if (ieq(tk.text, "NOT")) tk.t = Tok::Not;
                else if (ieq(tk.text, "TRUE")) { tk.t = Tok::Number; tk.num = 1; }
                else if (ieq(tk.text, "FALSE")) { tk.t = Tok::Number; tk.num = 0; }
            }
            return tk;
        }
        if ((c == '$' || c == '@') && p_ + 1 < s_.size() && is_alpha(s_[p_ + 1])) {
            size_t b = p_;
            ++p_;
            while (p_ < s_.size() && is_ident(s_[p_])) ++p_;
            col_ += (int)(p_ - b);
            tk.text.assign(s_, b, p_ - b);
            tk.t = c == '$' ? Tok::Var : Tok::Alias;
            return tk;
        }
        bool digit = is_digit(c);
        bool dot_digit = c == '.' && p_ + 1 < s_.size() && is_digit(s_[p_ + 1]);
        if (digit || dot_digit) return number(tk);
        auto two = [&](char a, char b) { return c == a && p_ + 1 < s_.size() && s_[p_ + 1] == b; };
        auto emit = [&](Tok t, int len) {  // operators and punctuation: no newline inside
            tk.t = t;
            tk.text.assign(s_, p_, len);
            p_ += len;
            col_ += len;
            return tk;
        };
        if (two('&', '&')) return emit(Tok::And, 2);
        if (two('|', '|')) return emit(Tok::Or, 2);
        if (two('=', '=')) return emit(Tok::Eq, 2);
        if (two('!', '=')) return emit(Tok::Ne, 2);
        if (two('<', '=')) return emit(Tok::Le, 2);
        if (two('>', '=')) return emit(Tok::Ge, 2);
        switch (c) {
            case '-': return emit(Tok::Minus, 1);
            case '+': return emit(Tok::Plus, 1);
            case '*': return emit(Tok::Star, 1);
            case '/': return emit(Tok::Slash, 1);
            case '(': return emit(Tok::LParen, 1);
            case ')': return emit(Tok::RParen, 1);
            case '=': return emit(Tok::Assign, 1);
            case '?': return emit(Tok::Question, 1);
            case ':': return emit(Tok::Colon, 1);
            case '&': return emit(Tok::And, 1);
            case '|': return emit(Tok::Or, 1);
            case '^': return emit(Tok::Xor, 1);
            case '!': return emit(Tok::Not, 1);
            case '<': return emit(Tok::Lt, 1);
            case '>': return emit(Tok::Gt, 1);
            case '{': return emit(Tok::LBrace, 1);
            case '}': return emit(Tok::RBrace, 1);
            case '.': return emit(Tok::Dot, 1);
            case ';': return emit(Tok::Semi, 1);
            case '[': return emit(Tok::LBracket, 1);
            case ']': return emit(Tok::RBracket, 1);
            case ',': return emit(Tok::Comma, 1);
            default: break;
        }
        fail(line_, col_, std::string("invalid character: ") + c);
    }

private:
    void adv() {
        if (s_[p_] == '\n') {
            ++line_;
            col_ = 1;
        } else {
            ++col_;
        }
        ++p_;
    }

    void skip() {
        while (p_ < s_.size()) {
            char c = s_[p_];
            if (c == ' ' || c == '\t' || c == '\r' || c == '\n') {
                adv();
            } else if (c == '/' && p_ + 1 < s_.size() && s_[p_ + 1] == '/') {
                while (p_ < s_.size() && s_[p_] != '\n') adv();
            } else {
                break;
            }
        }
    }

    Token number(Token tk) {
        size_t b = p_;
        bool is_float = false;
        while (p_ < s_.size() && is_digit(s_[p_])) ++p_;
        if (p_ < s_.size() && s_[p_] == '.') {
            is_float = true;
            ++p_;
            while (p_ < s_.size() && is_digit(s_[p_])) ++p_;
        }
        if (p_ < s_.size() && (s_[p_] == 'e' || s_[p_] == 'E')) {
            size_t q = p_ + 1;
            if (q < s_.size() && (s_[q] == '+' || s_[q] == '-')) ++q;
            if (q < s_.size() && is_digit(s_[q])) {
                is_float = true;
                p_ = q;
                while (p_ < s_.size() && is_digit(s_[p_])) ++p_;
            }
        }
        col_ += (int)(p_ - b);
        tk.text.assign(s_, b, p_ - b);
        errno = 0;
        if (is_float) {
            tk.t = Tok::Float;
            tk.num = std::strtod(tk.text.c_str(), nullptr);
            if (errno == ERANGE) fail(tk.line, tk.col, "float is out of range: " + tk.text);
        } else {
            tk.t = Tok::Number;
            long long v = std::strtoll(tk.text.c_str(), nullptr, 10);
            if (errno == ERANGE || v > INT_MAX) fail(tk.line, tk.col, "integer is out of range: " + tk.text);
            tk.num = (double)v;
        }
        return tk;
    }

    const std::string& s_;
    std::string f_;
    size_t p_ = 0;
    int line_ = 1, col_ = 1;
};

const char* tok_name(Tok t) {
    switch (t) {
        case Tok::Eof: return "end of file";
        case Tok::Ident: return "identifier";
        case Tok::Var: return "variable";
        case Tok::Alias: return "alias";
        case Tok::Number: return "integer";
        case Tok::Float: return "float";
        case Tok::Assign: return "\"=\"";
        case Tok::Semi: return "\";\"";
        case Tok::LBrace: return "\"{\"";
        case Tok::RBrace: return "\"}\"";
        case Tok::Dot: return "\".\"";
        case Tok::Colon: return "\":\"";
        case Tok::RParen: return "\")\"";
        case Tok::LBracket: return "\"[\"";
        case Tok::RBracket: return "\"]\"";
        case Tok::Comma: return "\",\"";
        default: return "operator";
    }
}

// Binding levels, lowest first (parser.yy:126-134).
enum Level { L_TERN = 1, L_XOR, L_OR, L_AND, L_EQ, L_REL, L_ADD, L_MUL, L_UNARY };

class Parser {
public:
    Parser(Model& m, const std::string& text, const std::string& fname) : m_(m), lx_(text, fname) {
        cur_ = lx_.next();
    }

    void bnd() {
        while (cur_.t != Tok::Eof) {
            Token kw = expect(Tok::Ident);
            if (!ieq(kw.text, "node")) lx_.fail(kw.line, kw.col, "expected 'node' keyword");
            Token name = expect(Tok::Ident);
            expect(Tok::LBrace);
            std::vector<std::pair<std::string, ExprPtr>> attrs;
            do {
                Token an = expect(Tok::Ident);
                expect(Tok::Assign);
                ExprPtr e = expr(L_TERN);
                expect(Tok::Semi);
                attrs.emplace_back(an.text, std::move(e));
            } while (cur_.t != Tok::RBrace);
            expect(Tok::RBrace);
            register_node(name, std::move(attrs));
        }
    }

    void cfg() {
        while (cur_.t != Tok::Eof) {
            if (cur_.t == Tok::Var) {
                Token v = take();
                expect(Tok::Assign);
                ExprPtr e = expr(L_TERN);
                expect(Tok::Semi);
                m_.variables[v.text] = guarded_eval(*e, v);
            } else if (cur_.t == Tok::LBracket) {
                istate_form();
            } else {
                Token id = expect(Tok::Ident);
                if (cur_.t == Tok::Dot) {
                    take();
                    Token attr = expect(Tok::Ident);
                    expect(Tok::Assign);
                    ExprPtr e = expr(L_TERN);
                    expect(Tok::Semi);
                    int ni = m_.node_index(id.text);
                    if (ni < 0) lx_.fail(id.line, id.col, "Unknown node " + id.text);
                    if (attr.text == "istate")
                        m_.nodes[ni].istate = guarded_eval(*e, attr);
                    else
                        m_.nodes[ni].attrs.emplace_back(attr.text, std::move(e));
                } else {
                    expect(Tok::Assign);
                    ExprPtr e = expr(L_TERN);
                    expect(Tok::Semi);
                    m_.constants[id.text] = guarded_eval(*e, id);
                }
            }
        }
    }

private:
    // `[A].istate = p [1], q [0];`  (parser.yy:102-108, driver.cpp:79-99)
    void istate_form() {
        expect(Tok::LBracket);
        Token node = expect(Tok::Ident);
        expect(Tok::RBracket);
        expect(Tok::Dot);
        Token attr = expect(Tok::Ident);
        if (attr.text != "istate") lx_.fail(attr.line, attr.col, "expected 'istate' keyword");
        expect(Tok::Assign);
        ExprPtr el = expr(L_TERN);
        expect(Tok::LBracket);
        Token nl = expect(Tok::Number);
        expect(Tok::RBracket);
        expect(Tok::Comma);
        ExprPtr er = expr(L_TERN);
        expect(Tok::LBracket);
        Token nr = expect(Tok::Number);
        expect(Tok::RBracket);
        expect(Tok::Semi);
        if (!((nl.num == 0 && nr.num == 1) || (nl.num == 1 && nr.num == 0)))
            lx_.fail(nl.line, nl.col, "numbers in [] must be 0 and 1");
        int ni = m_.node_index(node.text);
        if (ni < 0) lx_.fail(node.line, node.col, "Unknown node " + node.text);
        double l = guarded_eval(*el, node), r = guarded_eval(*er, node);
        m_.nodes[ni].istate = nl.num == 1 ? l / (l + r) : r / (l + r);
    }

    void register_node(const Token& name, std::vector<std::pair<std::string, ExprPtr>> attrs) {
        // driver.cpp:49-63
        if (m_.node_index(name.text) >= 0) lx_.fail(name.line, name.col, "Node " + name.text + " already exists");
        Node n;
        n.name = name.text;
        n.attrs = std::move(attrs);
        if (!n.attr("rate_up"))
            lx_.fail(name.line, name.col, "Node " + name.text + " does not have rate_up attribute");
        if (!n.attr("rate_down"))
            lx_.fail(name.line, name.col, "Node " + name.text + " does not have rate_down attribute");
        if ((int)m_.nodes.size() >= kMaxNodes) lx_.fail(name.line, name.col, "too many nodes");
        m_.add_node(std::move(n));
    }

    double guarded_eval(const Expr& e, const Token& at) {
        try {
            return eval_const(e, m_);
        } catch (const Error& err) {
            lx_.fail(at.line, at.col, err.what());
        }
    }

    Token take() {
        Token t = std::move(cur_);
        cur_ = lx_.next();
        return t;
    }

    [[noreturn]] __attribute__((noinline)) void unexpected(Tok want) const {
        lx_.fail(cur_.line, cur_.col,
                 std::string("syntax error, unexpected ") + tok_name(cur_.t) +
                     (cur_.text.empty() ? "" : " '" + cur_.text + "'") + ", expecting " + tok_name(want));
    }

    Token expect(Tok t) {
        if (cur_.t != t) unexpected(t);
        return take();
    }

    static int binary_level(Tok t, Op& op) {
        switch (t) {
            case Tok::Xor: op = Op::Xor; return L_XOR;
            case Tok::Or: op = Op::Or; return L_OR;
            case Tok::And: op = Op::And; return L_AND;
            case Tok::Eq: op = Op::Eq; return L_EQ;
            case Tok::Ne: op = Op::Ne; return L_EQ;
            case Tok::Lt: op = Op::Lt; return L_REL;
            case Tok::Le: op = Op::Le; return L_REL;
            case Tok::Gt: op = Op::Gt; return L_REL;
            case Tok::Ge: op = Op::Ge; return L_REL;
            case Tok::Plus: op = Op::Plus; return L_ADD;
            case Tok::Minus: op = Op::Minus; return L_ADD;
            case Tok::Star: op = Op::Star; return L_MUL;
            case Tok::Slash: op = Op::Slash; return L_MUL;
            default: return 0;
        }
    }

    ExprPtr primary() {
        auto mk = [](Expr::Kind k) {
            auto e = std::make_unique<Expr>();
            e->kind = k;
            return e;
        };
        switch (cur_.t) {
            case Tok::Number:
            case Tok::Float: {
                auto e = mk(Expr::Kind::Literal);
                e->value = cur_.num;
                take();
                return e;
            }
            case Tok::Ident:
            case Tok::Var:
            case Tok::Alias: {
                auto e = mk(cur_.t == Tok::Ident ? Expr::Kind::Ident
                                                 : cur_.t == Tok::Var ? Expr::Kind::Var : Expr::Kind::Alias);
                e->name = std::move(cur_.text);
                take();
                return e;
            }
            case Tok::LParen: {
                take();
                auto e = mk(Expr::Kind::Paren);
                e->a = expr(L_TERN);
                expect(Tok::RParen);
                return e;
            }
            case Tok::Minus:
            case Tok::Plus:
            case Tok::Not: {
                auto e = mk(Expr::Kind::Unary);
                e->op = cur_.t == Tok::Minus ? Op::Minus : cur_.t == Tok::Plus ? Op::Plus : Op::Not;
                take();
                e->a = expr(L_UNARY);
                return e;
            }
            default:
                lx_.fail(cur_.line, cur_.col,
                         std::string("syntax error, unexpected ") + tok_name(cur_.t) +
                             (cur_.text.empty() ? "" : " '" + cur_.text + "'"));
        }
    }

    ExprPtr expr(int min_level) {
        ExprPtr lhs = primary();
        for (;;) {
            if (cur_.t == Tok::Question) {
                if (L_TERN < min_level) break;
                take();
                auto e = std::make_unique<Expr>();
                e->kind = Expr::Kind::Ternary;
                e->a = std::move(lhs);
                e->b = expr(L_TERN);
                expect(Tok::Colon);
                e->c = expr(L_TERN);  // right associative
                lhs = std::move(e);
                continue;
            }
            Op op;
            int lvl = binary_level(cur_.t, op);
            if (lvl == 0 || lvl < min_level) break;
            take();
            auto e = std::make_unique<Expr>();
            e->kind = Expr::Kind::Binary;
            e->op = op;
            e->a = std::move(lhs);
            e->b = expr(lvl + 1);  // left associative
            lhs = std::move(e);
        }
        return lhs;
    }

    Model& m_;
    Lexer lx_;
    Token cur_;
};

}  // namespace

void parse_bnd(Model& m, const std::string& text, const std::string& fname) { Parser(m, text, fname).bnd(); }

void parse_cfg(Model& m, const std::string& text, const std::string& fname) { Parser(m, text, fname).cfg(); }

std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error("cannot open " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

}  // namespace mbg
