"""Shared helpers of the test suite: device runs, oracle runs and their comparison."""
from __future__ import annotations

import json
import os

import numpy as np

import oracle
import upmabossg_gb300 as mbg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TWO32 = 4294967296.0


def golden_model(name):
    with open(os.path.join(GOLDEN, "models", name + ".bnd")) as f:
        bnd = f.read()
    with open(os.path.join(GOLDEN, "models", name + ".cfg")) as f:
        cfg = f.read()
    return bnd, cfg


def golden_result(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def run_device(bnd, cfg, n_traj, layout=mbg.LAYOUT_AUTO, seed=None, record=True, **kw):
    model = mbg.Model.from_strings(bnd, cfg)
    sim = mbg.Simulation(model, n_traj=n_traj, layout=layout, seed=seed, record_trajectories=record, **kw)
    sim.run()
    return model, sim


def run_oracle(bnd, cfg, model, n_traj, seed=None, **kw):
    """The oracle on the same texts. It derives its fixed-point scale on its own (frac_bits 0), so a
    scale the product got wrong shows as differing trajectories; `model` (the product's parse) is
    not passed to it."""
    return oracle.run(bnd, cfg, frac_bits=0, n_traj=n_traj, seed=seed,
                      keep_trajectories=True, **kw)


def compare_trajectories(sim, orc, max_tie_frac=0.01):
    """Per-trajectory parity: states, statuses and transition counts bit-exact, end times within
    1e-5 relative, for every trajectory the oracle does not flag as a tie. Returns the tie count."""
    st, t, tr, status = sim.trajectories()
    ties = orc.ties != 0
    n_ties = int(ties.sum())
    assert n_ties <= max(1, max_tie_frac * len(ties)), f"{n_ties} ties in {len(ties)} trajectories"
    ok = ~ties
    bad = np.nonzero(ok & (status != orc.status))[0]
    assert bad.size == 0, f"status differs for trajectories {bad[:10]}: dev {status[bad[:10]]} orc {orc.status[bad[:10]]}"
    bad = np.nonzero(ok & (tr != orc.transitions))[0]
    assert bad.size == 0, f"transitions differ for {bad[:10]}: dev {tr[bad[:10]]} orc {orc.transitions[bad[:10]]}"
    bad = np.nonzero(ok & np.any(st != orc.states, axis=1))[0]
    assert bad.size == 0, f"end states differ for trajectories {bad[:10]}"
    rel = np.abs(t - orc.times) / np.maximum(np.abs(orc.times), 1e-30)
    assert float(rel[ok].max(initial=0)) <= 1e-5, f"end times differ: max rel {rel[ok].max()}"
    return n_ties


def sparse_th_raw(sim):
    """Raw TH sums without the dense window array (which is windows x 2^outputs)."""
    TH = np.zeros(sim.model.info.windows, np.uint64)
    mbg._check(mbg.lib().mbg_sim_probtraj_raw(sim._h, None, mbg._p(TH)))
    return None, TH


def compare_histograms(model, sim, orc, n_traj):
    """Window sums within 1e-5 x n x tick (time units), TH within 1e-4 relative, final states
    and fixed points exact up to tied trajectories."""
    info = model.info
    bins, sums, _ = sim.probtraj_sparse()
    _, th_raw = sparse_th_raw(sim)
    dev = sums.astype(np.float64) / (1.0 if info.discrete_time else TWO32)
    obins = (orc.hist_window.astype(np.uint64) << np.uint64(info.outputs)) | orc.hist_state.astype(np.uint64)
    keys = np.union1d(bins, obins)
    d = np.zeros(keys.size)
    r = np.zeros(keys.size)
    d[np.searchsorted(keys, bins)] = dev
    np.add.at(r, np.searchsorted(keys, obins), orc.hist_value)
    scale = n_traj * (1.0 if info.discrete_time else info.time_tick)
    n_ties = int((orc.ties != 0).sum())
    tol = 1e-5 * scale + (n_ties + 1) * (1.0 if info.discrete_time else info.time_tick) * 1.01
    err = float(np.abs(d - r).max(initial=0.0))
    assert err <= tol, f"window sums differ by {err} (tol {tol})"
    th_dev = th_raw.astype(np.float64) / TWO32
    th_err = np.abs(th_dev - orc.th)
    assert np.all(th_err <= 1e-4 * np.abs(orc.th) + 1e-4 * scale + n_ties * scale / n_traj * 5), \
        f"TH sums differ: max {th_err.max()}"
    fin = np.rint(sim.final_states() * n_traj)
    assert np.abs(fin - orc.final).sum() <= 2 * n_ties, "final-state histograms differ"
    fp_states, fp_probs = sim.fixed_points()
    ofix = orc.states[orc.status == 2]
    if ofix.size:
        uo, co = np.unique(ofix, axis=0, return_counts=True)
    else:
        uo, co = np.zeros((0, info.words), np.uint32), np.zeros(0, np.int64)
    if n_ties == 0:
        assert len(fp_states) == len(uo), f"{len(fp_states)} fixed points on the device, {len(uo)} in the oracle"
        dev_map = {tuple(s): int(round(p * n_traj)) for s, p in zip(fp_states, fp_probs)}
        orc_map = {tuple(s): int(c) for s, c in zip(uo, co)}
        assert dev_map == orc_map, "fixed points differ"
    return err


def mixed_network(n=48, seed=3, outputs=6, max_time=20.0, tick=0.5, discrete=False):
    """A random network exercising every rate form of the grammar: two-valued `@logic` rates,
    multi-valued (palette) rates that read other nodes (arithmetic on node values, nested ternaries,
    comparisons), XOR and NOT in the logic, constant nodes, and nodes with more than 12 regulators
    (stored outside the inline records). Returns (bnd, cfg)."""
    rng = np.random.default_rng(seed)
    names = [f"M{i}" for i in range(n)]
    lines = []
    for i, nm in enumerate(names):
        others = [x for x in names if x != nm]
        kind = i % 6
        if i == n - 1:  # a wide two-valued node: 14 regulators, beyond the 12 inline ones
            kind = 0
            regs = list(rng.choice(others, size=14, replace=False))
            logic = " | ".join(f"({a} & !{b})" for a, b in zip(regs[0::2], regs[1::2]))
        else:
            k = int(rng.integers(1, 4))
            regs = list(rng.choice(others, size=k, replace=False))
            ops = [" & ", " | ", " ^ "]
            logic = regs[0] if rng.random() < 0.5 else f"!{regs[0]}"
            for r in regs[1:]:
                logic = f"({logic}{ops[int(rng.integers(0, 3))]}{r})"
        u = float(np.round(rng.lognormal(0.0, 0.5), 4))
        d = float(np.round(rng.lognormal(0.0, 0.5), 4))
        a, b, c = rng.choice(others, size=3, replace=False)
        if kind == 0:
            up, down = f"@logic ? {u} : 0", f"@logic ? 0 : {d}"
        elif kind == 1:  # palette: the up rate scales with two other nodes
            up, down = f"@logic ? {u} * (1 + {a} + 2 * {b}) : 0", f"@logic ? 0 : {d}"
        elif kind == 2:  # palette: nested ternary on other nodes in the down rate
            up, down = f"@logic ? {u} : 0", f"@logic ? 0 : ({a} ? {d} : ({b} ? {2 * d} : {0.5 * d}))"
        elif kind == 3:  # palette: a comparison
            up, down = f"@logic ? ({a} + {b} + {c} >= 2 ? {2 * u} : {u}) : 0", f"@logic ? 0 : {d}"
        elif kind == 4 and i % 12 == 4:  # constant node (fixed points become common)
            logic = "1" if rng.random() < 0.5 else "0"
            up, down = f"@logic ? {u} : 0", f"@logic ? 0 : {d}"
        elif kind == 4:
            up, down = f"@logic ? {u} : 0", f"@logic ? 0 : {d}"
        else:
            up, down = f"@logic ? {u} : 0", f"@logic ? 0 : {d} * (2 - {a})"
        lines.append(f"Node {nm} {{\n  logic = {logic};\n  rate_up = {up};\n  rate_down = {down};\n}}\n")
    bnd = "".join(lines)
    out = set(rng.choice(names, size=outputs, replace=False))
    cfg = "".join(f"{nm}.is_internal = {0 if nm in out else 1};\n" for nm in names)
    cfg += "".join(f"{nm}.istate = 0.5;\n" for nm in names)
    cfg += f"max_time = {max_time};\ntime_tick = {tick};\nsample_count = 2000;\nseed_pseudorandom = 11;\n"
    if discrete:
        cfg += "discrete_time = 1;\n"
    return bnd, cfg
