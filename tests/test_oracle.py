"""Pins the oracle before it is trusted: Philox known answers, conservation laws, and the
reference's own golden outputs (test/*.res, decoded into tests/golden/*.json) within 4-sigma
binomial bounds."""
import math

import numpy as np
import pytest

import oracle
import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import golden_model, golden_result

# Random123 known-answer vectors for philox4x32-10 (Salmon et al., SC'11).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expected", KAT)
def test_philox_known_answers(ctr, key, expected):
    assert tuple(int(x) for x in oracle.philox(ctr, key)) == expected


def names_key(names, bits_in_node_order):
    return "|".join(n for n, b in zip(names, bits_in_node_order) if b)


def out_key(model, idx):
    return "|".join(model.names[o] for q, o in enumerate(model.outputs) if (idx >> q) & 1)


def full_key(model, words):
    n = model.info.nodes
    return "|".join(model.names[i] for i in range(n) if (int(words[i >> 5]) >> (i & 31)) & 1)


def sigma(p, n1, n2):
    return math.sqrt(max(p * (1 - p), 1.0 / min(n1, n2)) * (1.0 / n1 + 1.0 / n2))


def test_window_time_is_conserved():
    """Continuous time: every trajectory covers [0, max_time], so each full window holds n x tick
    of time and the final-state histogram counts every trajectory."""
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg(sample_count=64)
    m = mbg.Model.from_strings(bnd, cfg)
    r = oracle.run(bnd, cfg, frac_bits=m.info.frac_bits, n_traj=64, keep_trajectories=True)
    h = r.dense_hist()
    assert np.allclose(h.sum(axis=1), 64 * net.time_tick, rtol=1e-12)
    assert r.final.sum() == 64
    assert r.counters["pick_ties"] == 0
    assert np.all((r.status == 1) | (r.status == 2))
    assert np.all(r.times == net.max_time)


def test_fixed_point_states_have_zero_rate():
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg(sample_count=128)
    m = mbg.Model.from_strings(bnd, cfg)
    r = oracle.run(bnd, cfg, frac_bits=m.info.frac_bits, n_traj=128, keep_trajectories=True)
    fixed = r.states[r.status == 2]
    assert len(fixed) > 0
    for words in fixed[:5]:
        bits = [(int(words[i >> 5]) >> (i & 31)) & 1 for i in range(m.info.nodes)]
        assert all(m.rate(i, bits)[0] == 0 for i in range(m.info.nodes))


@pytest.mark.parametrize("name,n", [("cellcycle", 100000), ("sizek", 3000), ("metastasis", 4000),
                                    ("montagud", 4000)])
def test_oracle_matches_reference_goldens(name, n):
    bnd, cfg = golden_model(name)
    gold = golden_result(name)
    m = mbg.Model.from_strings(bnd, cfg)
    n_ref = m.info.sample_count
    # the goldens' final points come from an earlier build that flipped once more at the end
    r = oracle.run(bnd, cfg, frac_bits=m.info.frac_bits, n_traj=n, keep_trajectories=True, legacy_final=True)
    worst = 0.0

    def check(p_ref, p_orc, what):
        nonlocal worst
        s = sigma(0.5 * (p_ref + p_orc), n_ref, n)
        z = abs(p_ref - p_orc) / s
        worst = max(worst, z)
        assert z <= 4.0, f"{name} {what}: reference {p_ref} oracle {p_orc} ({z:.1f} sigma)"

    # final points (final_states.cpp:53-66)
    orc_final = {out_key(m, i): c / n for i, c in enumerate(r.final) if c}
    for k in set(gold["final"]) | set(orc_final):
        check(gold["final"].get(k, 0.0), orc_final.get(k, 0.0), f"final {k!r}")
    # fixed points: total mass and the most likely states (fixed_states.cu:139-152)
    fixed = r.states[r.status == 2]
    orc_fixed = {}
    for w in fixed:
        k = full_key(m, w)
        orc_fixed[k] = orc_fixed.get(k, 0) + 1
    check(gold["fixed_total"], len(fixed) / n, "fixed-point mass")
    for k, p in gold["fixed"].items():
        if p >= 0.01:
            check(p, orc_fixed.get(k, 0) / n, f"fixed {k[:40]!r}")
    # windows (window_average_small.cpp:142-179)
    h = r.dense_hist()
    scale = n if m.info.discrete_time else n * m.info.time_tick
    for wg in gold["windows"]:
        w = int(round(wg["start"] / m.info.time_tick))
        probs = h[w] / scale
        orc = {out_key(m, i): float(p) for i, p in enumerate(probs) if p > 0}
        for k in set(wg["probs"]) | set(orc):
            check(wg["probs"].get(k, 0.0), orc.get(k, 0.0), f"window {w} {k!r}")
        ent = -sum(p * math.log2(p) for p in orc.values() if p > 0)
        assert abs(ent - wg["entropy"]) <= 0.05 + 0.02 * wg["entropy"], f"{name} window {w} entropy"
        th = r.th[w] / scale
        assert abs(th - wg["th"]) <= 0.05 + 0.05 * wg["th"], f"{name} window {w} TH {th} vs {wg['th']}"
    print(f"{name}: worst deviation {worst:.2f} sigma")


def test_mlp_oracle_gradient_matches_finite_differences():
    from oracle import mlp
    rng = np.random.default_rng(3)
    dims = [5, 7, 6, 4]
    p = mlp.init_params(dims, rng).astype(np.float64)
    x = rng.normal(size=(9, 5))
    y = rng.dirichlet(np.ones(4), size=9)
    loss, g = mlp.loss_and_grad(p, dims, x, y, bf16=False)
    eps = 1e-6
    for i in rng.choice(len(p), 25, replace=False):
        q = p.copy()
        q[i] += eps
        lp, _ = mlp.loss_and_grad(q, dims, x, y, bf16=False)
        q[i] -= 2 * eps
        lm, _ = mlp.loss_and_grad(q, dims, x, y, bf16=False)
        assert abs((lp - lm) / (2 * eps) - g[i]) <= 1e-6 + 1e-5 * abs(g[i])


def test_bf16_rounding_is_nearest_even():
    from oracle import mlp
    assert mlp.bf16_round(np.float32(1.0)) == 1.0
    assert mlp.bf16_round(np.float32(1.0 + 2 ** -8)) == 1.0          # tie -> even
    assert mlp.bf16_round(np.float32(1.0 + 3 * 2 ** -8)) == 1.0 + 2 ** -6
    assert mlp.bf16_round(np.float32(-2.5)) == -2.5


@pytest.mark.parametrize("which", ["small", "medium", "mixed", "cellcycle", "montagud"])
def test_oracle_front_end_agrees_with_the_product_tables(which):
    """The oracle parses, evaluates and scales on its own (it shares no code with the product): the
    fixed-point scale it derives (frac_bits 0) gives the same trajectories as the product's."""
    from helpers import golden_model, mixed_network
    if which in ("small", "medium"):
        net = getattr(synth, which)()
        bnd, cfg = net.bnd(), net.cfg(sample_count=64)
    elif which == "mixed":
        bnd, cfg = mixed_network(seed=3)
    else:
        bnd, cfg = golden_model(which)
    m = mbg.Model.from_strings(bnd, cfg)
    a = oracle.run(bnd, cfg, n_traj=48, keep_trajectories=True)
    b = oracle.run(bnd, cfg, frac_bits=m.info.frac_bits, n_traj=48, keep_trajectories=True)
    assert np.array_equal(a.states, b.states) and np.array_equal(a.transitions, b.transitions)
    assert np.array_equal(a.times, b.times)
