// Model front-end: AST, parsed model and the compiled (table) form used by the kernels.
//
// The grammar and the evaluation rules restate the reference's front-end:
//   tokens            src/parser/scanner.ll:51-94
//   grammar           src/parser/parser.yy:74-158 (precedence 126-134)
//   driver semantics  src/parser/driver.cpp:7-99, src/parser/parse_types.cpp:3-23
//   expression rules  src/parser/expressions.cpp:10-231
// Differences, all deliberate: expressions evaluate in double (the reference uses float), XOR
// is supported (the reference throws, expressions.cpp:79,148), and the `[A].istate = p [1], q [0];`
// form lexes (the reference scanner has no `[`, `]` or `,` tokens).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace mbg {

enum class Op { Plus, Minus, Star, Slash, And, Or, Xor, Not, Le, Lt, Ge, Gt, Eq, Ne };

struct Expr;
using ExprPtr = std::unique_ptr<Expr>;

struct Expr {
    enum class Kind { Literal, Ident, Var, Alias, Unary, Binary, Ternary, Paren };
    Kind kind;
    double value = 0.0;  // Literal
    std::string name;    // Ident, Var ("$x"), Alias ("@x")
    Op op = Op::Plus;    // Unary, Binary
    ExprPtr a, b, c;     // operands
};

class Error : public std::runtime_error {
public:
    explicit Error(const std::string& m) : std::runtime_error(m) {}
};

struct Node {
    std::string name;
    std::vector<std::pair<std::string, ExprPtr>> attrs;  // first match wins, as parse_types.cpp:8-13
    double istate = 0.5;                                 // parse_types.cpp:3

    const Expr* attr(const std::string& n) const;
};

struct Model {
    std::vector<Node> nodes;
    std::unordered_map<std::string, double> variables;  // "$name" -> value
    std::map<std::string, double> constants;  // defaults from driver.cpp:9-13

    std::unordered_map<std::string, int> index;  // node name -> position in `nodes`

    Model();
    int node_index(const std::string& name) const;  // -1 if unknown
    void add_node(Node&& n);                          // appends and indexes
    bool is_internal(int i) const;                   // parse_types.cpp:20-23
    double constant(const std::string& n) const;
};

// Parse a .bnd text then a .cfg text into `m` (driver.cpp:16-31). Throws mbg::Error with
// "<file>:<line>:<col>: message" on any syntax or semantic error.
void parse_bnd(Model& m, const std::string& text, const std::string& fname);
void parse_cfg(Model& m, const std::string& text, const std::string& fname);
std::string read_file(const std::string& path);

// Expression evaluation. `state` is indexed by node; `cur` is the node whose attributes
// @aliases resolve against (expressions.cpp:223-231).
double eval_const(const Expr& e, const Model& m);
double eval_state(const Expr& e, const Model& m, int cur, const uint8_t* state);
// Every node index an expression reads, with @aliases expanded for node `cur`.
void collect_support(const Expr& e, const Model& m, int cur, std::vector<int>& out, int depth = 0);

// ---------------------------------------------------------------------------------------------
// Compiled form. Rates are unsigned fixed point with `frac_bits` fraction bits so that sums,
// prefix scans and incremental updates are exact and order independent.

enum NodeKind : uint16_t {
    NODE_BINARY = 0,   // rate = bit(self, idx) ? (self ? down : up) : 0
    NODE_PALETTE = 1,  // rate = palette[pidx(self, idx)]
};

struct CompiledNode {
    std::vector<int> regs;         // support minus the node itself, ascending
    NodeKind kind = NODE_BINARY;
    std::vector<uint32_t> bits;    // NODE_BINARY: 2^(k+1) bits, bit (self<<k)|idx
    uint64_t up = 0, down = 0;     // NODE_BINARY fixed-point rates
    double up_real = 0, down_real = 0;
    std::vector<uint8_t> pidx;     // NODE_PALETTE: 2^(k+1) palette indices
    std::vector<uint64_t> palette; // NODE_PALETTE fixed-point values (palette[0] may be non-zero)
    std::vector<double> palette_real;
};

struct CompiledModel {
    int n = 0, words = 0, n_out = 0;
    int frac_bits = 32;
    std::vector<CompiledNode> nodes;
    std::vector<int> out_nodes;         // output (non-internal) nodes in node order
    std::vector<int> out_pos;           // per node: position among outputs or -1
    std::vector<double> istate;         // per node activation probability
    std::vector<uint32_t> istate_thr;   // per node 24-bit threshold: on iff (u32 >> 8) < thr
    std::vector<std::vector<int>> deps; // per node: nodes whose rate reads it, plus itself
    int max_k = 0;
    // run constants
    bool discrete = false;
    double max_time = 10, tick = 0.1;
    uint64_t sample_count = 1000000, seed = 0;
    int windows = 0;
};

// Limits of the compiled representation.
constexpr int kMaxBinaryRegs = 24;   // 2^25 table bits per node at most
constexpr int kMaxPaletteRegs = 12;  // 2^13 palette indices per node at most
constexpr int kMaxNodes = 65535;     // regulator indices are stored as uint16

CompiledModel compile_model(const Model& m);
// Copy of cm with node i's up rates times up_scale[i] and down rates times down_scale[i] (null:
// 1), fixed-point scale and quantisation redone by compile_model's rule. Throws for palette nodes.
CompiledModel rescale_model(const CompiledModel& cm, const double* up_scale, const double* down_scale);
// Copy of cm with node nodes[j] clamped to values[j] (1 ON, 0 OFF): its initial state is the value
// and its rate is zero wherever it holds the value. The fixed-point scale and the compiled form of
// every node are what compile_model gives for the model whose clamped nodes have `istate` the value
// and the opposite rate (rate_down for ON, rate_up for OFF) equal to 0.
CompiledModel mutate_model(const CompiledModel& cm, const int* nodes, const int* values, int count);
uint64_t quantize_rate(double r, int frac_bits);  // round-to-nearest, throws on overflow

// Run constants of a model (the cfg's max_time, time_tick, sample_count, seed_pseudorandom,
// discrete_time).
struct RunConstants {
    double max_time = 10, tick = 0.1;
    uint64_t sample_count = 1000000, seed = 0;
    bool discrete = false;
};
// A model given by arrays instead of text. Node i reads regs[reg_off[i] .. reg_off[i + 1])
// (distinct node indices other than i, in any order); its logic over them is bit
// idx = sum_j state(regs[reg_off[i] + j]) << j of the words logic[logic_off[i] ..] (within the
// logic_words words of `logic`); it turns on at
// rate_up[i] while off with logic 1 and off at rate_down[i] while on with logic 0 (the MaBoSS
// form `rate_up = @logic ? u : 0; rate_down = @logic ? 0 : d;`, which compile_model tabulates
// the same way); istate[i] in [0, 1]; an output iff is_output[i] (null: every node). The
// fixed-point scale and quantisation follow compile_model's rule. Throws Error on bad input.
CompiledModel compile_arrays(int n, const int32_t* reg_off, const int32_t* regs, const uint32_t* logic,
                             int64_t logic_words, const int64_t* logic_off, const double* rate_up,
                             const double* rate_down, const double* istate, const uint8_t* is_output,
                             const RunConstants& rc);

}  // namespace mbg
