"""Models built from arrays (mbg_model_from_arrays) against the same networks written as .bnd/.cfg
text: the compiled rates agree in every state, bad inputs are refused, and (on the GPU) the two
handles simulate identically."""
import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth


def random_table_network(seed, n=12, max_k=4, out_frac=0.6):
    """A random network given as regulator lists and truth tables, and the same network as a
    synth.Network whose logic is the truth table's minterm formula."""
    rng = np.random.default_rng(seed)
    names = [f"G{i}" for i in range(n)]
    regs, tabs, formulas = [], [], []
    for i in range(n):
        k = int(rng.integers(0, max_k + 1))
        r = [int(x) for x in rng.choice([j for j in range(n) if j != i], size=k, replace=False)]
        t = rng.integers(0, 2, size=1 << k).astype(np.uint8)
        terms = []
        for idx in range(1 << k):
            if t[idx]:
                lits = [(names[r[j]] if (idx >> j) & 1 else "!" + names[r[j]]) for j in range(k)]
                terms.append("(" + " & ".join(lits) + ")" if lits else "1")
        regs.append(r)
        tabs.append(t)
        # a table with no true entry still reads its regulators, as the array form does
        formulas.append(" | ".join(terms) if terms else
                        ("(" + " & ".join(names[x] for x in r) + ") & 0" if r else "0"))
    up = synth.round_rates(rng.lognormal(0, 0.5, n))
    down = synth.round_rates(rng.lognormal(0, 0.5, n))
    istate = np.array([float(f"{v:.6g}") for v in rng.uniform(0, 1, n)])
    outputs = sorted(int(x) for x in rng.choice(n, size=max(1, int(out_frac * n)), replace=False))
    net = synth.Network(names=names, logic=formulas, up=up, down=down, outputs=outputs, istate=istate,
                        sample_count=2000, max_time=8.0, time_tick=0.5, seed=11)
    is_out = np.zeros(n, np.uint8)
    is_out[outputs] = 1
    return net, regs, tabs, is_out


def both_models(seed, **kw):
    net, regs, tabs, is_out = random_table_network(seed, **kw)
    text = mbg.Model.from_strings(net.bnd(), net.cfg())
    arr = mbg.Model.from_arrays(regs, tabs, net.up, net.down, net.istate, is_output=is_out, names=net.names,
                                max_time=net.max_time, time_tick=net.time_tick, sample_count=net.sample_count,
                                seed=net.seed)
    return net, text, arr


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_arrays_compile_like_text(seed):
    net, text, arr = both_models(seed)
    for key in ("nodes", "words", "outputs", "windows", "frac_bits", "discrete_time", "sample_count", "seed"):
        assert getattr(text.info, key) == getattr(arr.info, key), key
    assert text.names == arr.names and text.outputs == arr.outputs
    rng = np.random.default_rng(seed)
    n = len(net.names)
    for _ in range(200):
        state = rng.integers(0, 2, size=n).astype(np.uint8)
        for i in range(n):
            assert text.rate(i, state) == arr.rate(i, state), (i, state)


def test_array_defaults():
    m = mbg.Model.from_arrays([[1], [0]], [[0, 1], [1, 0]], [1.0, 2.0], [0.5, 0.25], [0.5, 1.0])
    assert m.names == ["N0", "N1"] and m.outputs == [0, 1]
    # N0 copies N1: off with N1 on turns on at 1.0; N1 negates N0: on with N0 on turns off at 0.25
    assert m.rate(0, [0, 1])[1] == 1.0 and m.rate(0, [0, 0])[1] == 0.0
    assert m.rate(1, [1, 1])[1] == 0.25 and m.rate(1, [0, 1])[1] == 0.0


@pytest.mark.parametrize("case", ["self", "range", "twice", "table", "rate", "istate", "names"])
def test_bad_arrays_are_refused(case):
    regs, tabs = [[1], [0]], [[0, 1], [1, 0]]
    up, down, ist, names = [1.0, 1.0], [1.0, 1.0], [0.5, 0.5], None
    if case == "self":
        regs = [[0], [0]]
    elif case == "range":
        regs = [[5], [0]]
    elif case == "twice":
        regs, tabs = [[1, 1], [0]], [[0, 1, 1, 0], [1, 0]]
    elif case == "table":
        tabs = [[0, 1, 1], [1, 0]]
    elif case == "rate":
        up = [-1.0, 1.0]
    elif case == "istate":
        ist = [1.5, 0.5]
    elif case == "names":
        names = ["A", "A"]
    with pytest.raises((mbg.MbgError, ValueError)):
        mbg.Model.from_arrays(regs, tabs, up, down, ist, names=names)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [4, 5])
def test_arrays_simulate_like_text(seed):
    net, text, arr = both_models(seed, n=40, max_k=5)
    a = mbg.Simulation(text, n_traj=3000, seed=9).run()
    b = mbg.Simulation(arr, n_traj=3000, seed=9).run()
    assert np.array_equal(a.probtraj_raw()[0], b.probtraj_raw()[0])
    assert np.array_equal(a.probtraj_raw()[1], b.probtraj_raw()[1])
    assert np.array_equal(a.final_states(), b.final_states())
    fa, pa = a.fixed_points()
    fb, pb = b.fixed_points()
    assert np.array_equal(fa, fb) and np.array_equal(pa, pb)
    assert a.summary()["transitions"] == b.summary()["transitions"]


def test_truth_table_outside_the_logic_array_is_refused():
    """The C entry point checks every node's table against the length of `logic` it is given."""
    import ctypes
    from upmabossg_gb300 import lib, ModelRun
    reg_off = np.array([0, 1, 2], np.int32)
    regs = np.array([1, 0], np.int32)
    logic = np.array([0b10, 0b01], np.uint32)
    up, down, ist = (np.ones(2), np.ones(2), np.full(2, 0.5))
    run = ModelRun(10.0, 0.5, 100, 0, 0, 0)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for words, offs in ((2, [0, 1]), (1, [0, 1]), (2, [0, -1])):
        h = ctypes.c_void_p()
        off = np.array(offs, np.int64)  # held for the call
        st = lib().mbg_model_from_arrays(2, None, p(reg_off), p(regs), p(logic), words, p(off), p(up), p(down),
                                         p(ist), None, ctypes.byref(run), ctypes.byref(h))
        if words == 2 and offs == [0, 1]:
            assert st == 0
            lib().mbg_model_destroy(h)
        else:
            assert st != 0 and not h.value
