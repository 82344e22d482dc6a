"""Grammar and rate semantics of the model front-end (src/parser/scanner.ll, parser.yy,
driver.cpp, expressions.cpp), checked through the compiled per-node rate tables."""
import itertools
import math

import numpy as np
import pytest

import upmabossg_gb300 as mbg

from helpers import golden_model


def node_block(name, logic, up="@logic ? 1 : 0", down="@logic ? 0 : 1", extra=""):
    return f"Node {name} {{ logic = {logic}; rate_up = {up}; rate_down = {down}; {extra} }}\n"


def rates_of(model, node):
    """All (state tuple -> real rate) of one node over every state of a small model."""
    n = model.info.nodes
    out = {}
    for bits in itertools.product((0, 1), repeat=n):
        out[bits] = model.rate(node, bits)[1]
    return out


def check_logic(expr_text, pyfunc, names=("A", "B", "C")):
    """Node X's logic is `expr_text` over A, B, C; its rate must be 1 exactly when the
    logic differs from its own state (the @logic form of generator.cpp:93-107)."""
    bnd = "".join(node_block(n, n) for n in names) + node_block("X", expr_text)
    m = mbg.Model.from_strings(bnd, "")
    x = m.info.nodes - 1
    for bits, r in rates_of(m, x).items():
        logic = bool(pyfunc(*bits[:len(names)]))
        expected = 1.0 if logic != bool(bits[x]) else 0.0
        assert r == expected, f"{expr_text} at {bits}: {r} != {expected}"


def test_and_or_not_spellings():
    for a, o, n in (("&", "|", "!"), ("&&", "||", "!"), ("AND", "OR", "NOT"), ("and", "or", "not")):
        check_logic(f"{n} A {a} (B {o} C)", lambda A, B, C: (not A) and (B or C))


def test_precedence_and_binds_tighter_than_or():
    check_logic("A | B & C", lambda A, B, C: A or (B and C))


def test_precedence_xor_is_loosest():
    # parser.yy:126-134 lists XOR below OR: A | B ^ C == (A | B) ^ C
    check_logic("A | B ^ C", lambda A, B, C: (A or B) != C)
    check_logic("A ^ B & C", lambda A, B, C: A != (B and C))


def test_not_binds_tightest():
    check_logic("!A & B", lambda A, B, C: (not A) and B)
    check_logic("!(A & B)", lambda A, B, C: not (A and B))


def test_true_false_and_comparisons():
    check_logic("TRUE", lambda A, B, C: True)
    check_logic("false | A", lambda A, B, C: A)
    check_logic("A + B + C >= 2", lambda A, B, C: A + B + C >= 2)
    check_logic("A == B", lambda A, B, C: A == B)
    check_logic("A != B", lambda A, B, C: A != B)


def test_ternary_is_right_associative():
    check_logic("A ? B : C ? A : B", lambda A, B, C: B if A else (A if C else B))


def test_comments_and_case_insensitive_node_keyword():
    bnd = "// c\nnode A { logic = A; rate_up = @logic ? 1 : 0; rate_down = @logic ? 0 : 1; } // t\n" \
          "NODE B { logic = !A; rate_up = @logic ? 2 : 0; rate_down = @logic ? 0 : 3; }"
    m = mbg.Model.from_strings(bnd, "")
    assert m.names == ["A", "B"]
    assert m.rate(1, (0, 0))[1] == 2.0
    assert m.rate(1, (0, 1))[1] == 0.0
    assert m.rate(1, (1, 1))[1] == 3.0


def test_variables_and_float_forms():
    # B's logic is !A: B turns on at rate $u when A is off, off at rate $d when A is on
    bnd2 = node_block("A", "A") + node_block("B", "!A", up="@logic ? $u : 0", down="@logic ? 0 : $d")
    for lit, val in (("1.5", 1.5), (".25", 0.25), ("3.", 3.0), ("2e-1", 0.2), ("1.5E+1", 15.0), ("7", 7.0)):
        m = mbg.Model.from_strings(bnd2, f"$u = {lit}; $d = $u * 2;")
        assert m.rate(1, (0, 0))[1] == pytest.approx(val)
        assert m.rate(1, (1, 1))[1] == pytest.approx(2 * val)


def test_general_rate_expression_and_palette():
    # rate depends on other nodes beyond one logic bit: multi-valued (palette) node
    bnd = node_block("A", "A") + node_block("B", "B") + \
        "Node C { rate_up = 1 + A + 2 * B; rate_down = 0.5; }\n"
    m = mbg.Model.from_strings(bnd, "")
    assert m.info.palette_nodes == 1
    for a in (0, 1):
        for b in (0, 1):
            assert m.rate(2, (a, b, 0))[1] == 1 + a + 2 * b
            assert m.rate(2, (a, b, 1))[1] == 0.5


def test_alias_to_custom_attribute():
    bnd = node_block("A", "A") + \
        "Node B { logic = A; k = 4; rate_up = @logic ? @k : 0; rate_down = @logic ? 0 : @k / 2; }\n"
    m = mbg.Model.from_strings(bnd, "")
    assert m.rate(1, (1, 0))[1] == 4.0
    assert m.rate(1, (0, 1))[1] == 2.0


def test_cfg_attribute_cannot_override_bnd_attribute():
    # parse_types.cpp:8-13: attributes are looked up first-match, cfg appends after bnd
    bnd = node_block("A", "A") + node_block("B", "A", up="@logic ? 1 : 0")
    m = mbg.Model.from_strings(bnd, "B.rate_up = 5;")
    assert m.rate(1, (1, 0))[1] == 1.0


def test_is_internal_and_istate_forms():
    bnd = node_block("A", "A") + node_block("B", "B") + node_block("C", "C")
    cfg = "A.is_internal = 1; B.is_internal = FALSE; [C].istate = 3 [1], 1 [0]; A.istate = 0.25;"
    m = mbg.Model.from_strings(bnd, cfg)
    assert m.outputs == [1, 2]


def test_duplicate_node_is_an_error():
    with pytest.raises(mbg.MbgError):
        mbg.Model.from_strings(node_block("A", "A") + node_block("A", "A"), "")


def test_unknown_identifier_is_a_model_error():
    with pytest.raises(mbg.MbgError) as e:
        mbg.Model.from_strings(node_block("A", "Z"), "")
    assert "Z" in e.value.message


def test_invalid_character():
    with pytest.raises(mbg.MbgError) as e:
        mbg.Model.from_strings("Node A { logic = A # B; rate_up = 1; rate_down = 1; }", "")
    assert "invalid character" in e.value.message


def test_constants_and_defaults():
    m = mbg.Model.from_strings(node_block("A", "A"), "")
    assert m.info.max_time == 10 and m.info.time_tick == pytest.approx(0.1)
    assert m.info.sample_count == 1000000 and m.info.discrete_time == 0
    assert m.info.windows == 100
    m = mbg.Model.from_strings(node_block("A", "A"), "max_time = 5; time_tick = .2; discrete_time = 1; "
                                                     "sample_count = 12.0; seed_pseudorandom = 100;")
    assert m.info.windows == 25 and m.info.discrete_time == 1 and m.info.sample_count == 12
    assert m.info.seed == 100


@pytest.mark.parametrize("name,n,outs", [("cellcycle", 10, 4), ("metastasis", 32, 5), ("sizek", 87, 4),
                                         ("montagud", 133, 3)])
def test_reference_data_models_parse(name, n, outs):
    bnd, cfg = golden_model(name)
    m = mbg.Model.from_strings(bnd, cfg)
    assert m.info.nodes == n
    assert m.info.outputs == outs
    assert m.info.max_regulators <= 13
    assert m.info.palette_nodes == 0


def test_fixed_point_rate_quantisation():
    bnd = node_block("A", "!A", up="@logic ? 0.123456 : 0", down="@logic ? 0 : 7")
    m = mbg.Model.from_strings(bnd, "")
    q, r = m.rate(0, (0,))
    F = m.info.frac_bits
    assert r == 0.123456 and q == round(math.ldexp(0.123456, F))


class _Gen:
    """Random rate expressions over nodes A..E mixing logic, comparisons, arithmetic on node
    values and ternaries, as text and as a Python function of the node values (the grammar's
    double semantics: logical operators and comparisons give 1.0 or 0.0)."""

    NAMES = ("A", "B", "C", "D", "E")

    def __init__(self, rng):
        self.rng = rng

    def expr(self, depth):
        r = self.rng
        if depth == 0 or r.random() < 0.2:
            if r.random() < 0.7:
                i = int(r.integers(0, len(self.NAMES)))
                return self.NAMES[i], (lambda s, i=i: float(s[i]))
            c = float(r.choice([0.0, 1.0, 0.5, 2.0, 3.25]))
            return repr(c), (lambda s, c=c: c)
        kind = int(r.integers(0, 5))
        a, fa = self.expr(depth - 1)
        if kind == 0:  # NOT
            return f"!({a})", (lambda s, fa=fa: 1.0 if fa(s) == 0 else 0.0)
        b, fb = self.expr(depth - 1)
        if kind == 1:
            op = str(r.choice(["&", "|", "^"]))
            f = {"&": lambda x, y: x != 0 and y != 0, "|": lambda x, y: x != 0 or y != 0,
                 "^": lambda x, y: (x != 0) != (y != 0)}[op]
            return f"({a} {op} {b})", (lambda s, fa=fa, fb=fb, f=f: 1.0 if f(fa(s), fb(s)) else 0.0)
        if kind == 2:
            op = str(r.choice(["<", "<=", ">", ">=", "==", "!="]))
            f = {"<": lambda x, y: x < y, "<=": lambda x, y: x <= y, ">": lambda x, y: x > y,
                 ">=": lambda x, y: x >= y, "==": lambda x, y: x == y, "!=": lambda x, y: x != y}[op]
            return f"({a} {op} {b})", (lambda s, fa=fa, fb=fb, f=f: 1.0 if f(fa(s), fb(s)) else 0.0)
        if kind == 3:
            op = str(r.choice(["+", "-", "*"]))
            f = {"+": lambda x, y: x + y, "-": lambda x, y: x - y, "*": lambda x, y: x * y}[op]
            return f"({a} {op} {b})", (lambda s, fa=fa, fb=fb, f=f: f(fa(s), fb(s)))
        c, fc = self.expr(depth - 1)
        return f"({a} ? {b} : {c})", (lambda s, fa=fa, fb=fb, fc=fc: fb(s) if fa(s) != 0 else fc(s))


@pytest.mark.parametrize("seed", range(12))
def test_random_expressions_tabulate_exactly(seed):
    """Every node's rate table, built 64 assignments at a time, equals a direct evaluation of its
    rate expressions (squared plus a constant, so that every rate is positive and finite) for every
    state of the model, value for value."""
    g = _Gen(np.random.default_rng(seed))
    blocks, funcs = [], []
    for name in g.NAMES:
        up, fu = g.expr(4)
        down, fd = g.expr(4)
        blocks.append(node_block(name, "A", up=f"({up}) * ({up}) + 0.25", down=f"({down}) * ({down}) / 2 + 0.125"))
        funcs.append((fu, fd))
    m = mbg.Model.from_strings("".join(blocks), "")
    n = len(g.NAMES)
    for i in range(n):
        fu, fd = funcs[i]
        for bits in itertools.product((0, 1), repeat=n):
            want = fd(bits) * fd(bits) / 2 + 0.125 if bits[i] else fu(bits) * fu(bits) + 0.25
            assert m.rate(i, bits)[1] == want, (i, bits)


def test_compile_error_names_the_lowest_failing_node():
    """Nodes are tabulated on several host threads once a model has 256 or more; when several fail,
    the error is the one of the lowest-numbered node, as a single thread would have reported it."""
    n = 400
    names = [f"X{i}" for i in range(n)]
    bad = (150, 280, 390)  # each reads 25 nodes, one over the limit of 24
    lines = []
    for i, nm in enumerate(names):
        if i in bad:
            regs = [names[(i + 1 + j) % n] for j in range(25)]
            logic = " | ".join(regs)
        else:
            logic = f"!{names[(i + 1) % n]}"
        lines.append(f"Node {nm} {{ logic = {logic}; rate_up = @logic ? 1 : 0; rate_down = @logic ? 0 : 1; }}\n")
    cfg = "max_time = 5;\ntime_tick = 1;\nsample_count = 10;\n"
    for _ in range(3):  # the same error whichever thread reaches a bad node first
        with pytest.raises(mbg.MbgError) as e:
            mbg.Model.from_strings("".join(lines), cfg)
        assert "node X150 reads 25 nodes" in e.value.message, e.value.message
