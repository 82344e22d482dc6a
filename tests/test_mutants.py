"""Mutant analysis, cfg overrides and the final-state CSV.

A mutant (``mbg_model_with_mutations``) clamps nodes ON or OFF. It must simulate exactly as the
model written out in the reference's own language: the clamped node's ``istate`` set to the value
in the cfg and its ``rate_down`` (ON) or ``rate_up`` (OFF) set to 0 in the bnd. The CPU tests
compare the compiled rates of the two over every state; the GPU tests compare whole simulations
bit for bit, and the device's mutant run against the oracle on the rewritten model.
"""
import itertools
import os
import subprocess

import numpy as np
import pytest

import upmabossg_gb300 as mbg

from helpers import compare_histograms, compare_trajectories, run_oracle


def _node(name, logic, up, down):
    return f"Node {name} {{ logic = {logic}; rate_up = {up}; rate_down = {down}; }}\n"


# A binary node, a node with a variable, a node with multi-valued rates on both sides (palette
# form), and an internal node.
NODES = {
    "A": ("B AND NOT C", "@logic ? $ka : 0", "@logic ? 0 : 2.5"),
    "B": ("A OR C", "@logic ? 1.5 : 0", "@logic ? 0 : $kb"),
    "C": ("NOT A", "@logic ? (B ? 3 : 0.7) : 0", "@logic ? 0 : 1"),
    "D": ("A", "A ? 2 : 0.5", "B ? 3 : 0.25"),
    "E": ("D AND NOT B", "@logic ? 1 : 0", "@logic ? 0 : 4"),
}
CFG = ("$ka = 1.25; $kb = 0.75; max_time = 6; time_tick = 0.5; sample_count = 4000; seed_pseudorandom = 9;\n"
       "E.is_internal = 1;\n")


def _bnd(clamps=None):
    clamps = clamps or {}
    out = ""
    for name, (logic, up, down) in NODES.items():
        if clamps.get(name) == 1:
            down = "0"
        elif clamps.get(name) == 0:
            up = "0"
        out += _node(name, logic, up, down)
    return out


def _cfg(clamps=None):
    return CFG + "".join(f"{n}.istate = {v};\n" for n, v in (clamps or {}).items())


def _rates(model):
    n = model.info.nodes
    return {(i, bits): model.rate(i, bits)[0] for i in range(n) for bits in itertools.product((0, 1), repeat=n)}


CASES = [{"A": 1}, {"A": 0}, {"C": 0}, {"D": 0}, {"D": 1}, {"B": 1, "C": 0}, {"A": 0, "D": 1, "E": 1}]


@pytest.mark.parametrize("clamps", CASES, ids=lambda c: ",".join(f"{k}{v}" for k, v in c.items()))
def test_mutant_compiles_as_the_rewritten_model(clamps):
    base = mbg.Model.from_strings(_bnd(), _cfg())
    mutant = base.with_mutations({k: ("ON" if v else "OFF") for k, v in clamps.items()})
    rewritten = mbg.Model.from_strings(_bnd(clamps), _cfg(clamps))
    assert mutant.info.frac_bits == rewritten.info.frac_bits
    assert mutant.info.outputs == rewritten.info.outputs
    assert _rates(mutant) == _rates(rewritten)


def test_mutant_arguments_are_checked():
    base = mbg.Model.from_strings(_bnd(), _cfg())
    with pytest.raises(ValueError):
        base.with_mutations({"A": "UP"})
    with pytest.raises(mbg.MbgError):
        base.with_mutations({17: 1})
    with pytest.raises(mbg.MbgError):
        base.with_mutations({0: 2})
    # an empty mutation list is the base model
    assert _rates(base.with_mutations({})) == _rates(base)


def test_cfg_overrides_replace_cfg_values(tmp_path):
    (tmp_path / "m.bnd").write_text(_bnd())
    (tmp_path / "m.cfg").write_text(_cfg())
    over = mbg.Model.from_files(str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg"),
                                overrides="$ka = 3.5; max_time = 7; sample_count = 123;")
    edited = mbg.Model.from_strings(_bnd(), _cfg().replace("$ka = 1.25", "$ka = 3.5")
                                    .replace("max_time = 6", "max_time = 7").replace("4000", "123"))
    assert over.info.max_time == 7 and over.info.sample_count == 123
    assert _rates(over) == _rates(edited)
    with pytest.raises(mbg.MbgError):
        mbg.Model.from_files(str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg"), overrides="$ka = ;")


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [mbg.LAYOUT_THREAD, mbg.LAYOUT_WARP, mbg.LAYOUT_LANE])
@pytest.mark.parametrize("clamps", CASES[:4] + CASES[5:], ids=lambda c: ",".join(f"{k}{v}" for k, v in c.items()))
def test_mutant_simulates_as_the_rewritten_model(clamps, layout):
    base = mbg.Model.from_strings(_bnd(), _cfg())
    mutant = base.with_mutations(clamps)
    rewritten = mbg.Model.from_strings(_bnd(clamps), _cfg(clamps))
    a = mbg.Simulation(mutant, n_traj=4000, layout=layout, record_trajectories=True).run()
    b = mbg.Simulation(rewritten, n_traj=4000, layout=layout, record_trajectories=True).run()
    for x, y in zip(a.probtraj_raw(), b.probtraj_raw()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.final_states(), b.final_states())
    for x, y in zip(a.fixed_points(), b.fixed_points()):
        assert np.array_equal(x, y)
    for x, y in zip(a.trajectories(), b.trajectories()):
        assert np.array_equal(x, y)
    # a clamped output node holds its value in every window
    P, _ = a.probtraj()
    for name, v in clamps.items():
        i = mutant.names.index(name)
        if i in mutant.outputs:
            bit = mutant.outputs.index(i)
            held = np.array([((s >> bit) & 1) == v for s in range(P.shape[1])])
            assert np.allclose(P[:, held].sum(axis=1), 1.0, atol=1e-9)


@pytest.mark.gpu
def test_mutant_matches_the_oracle_on_the_rewritten_model():
    clamps = {"B": 1, "C": 0}
    base = mbg.Model.from_strings(_bnd(), _cfg())
    mutant = base.with_mutations(clamps)
    n = 4000
    sim = mbg.Simulation(mutant, n_traj=n, record_trajectories=True).run()
    orc = run_oracle(_bnd(clamps), _cfg(clamps), mutant, n)
    compare_trajectories(sim, orc)
    compare_histograms(mutant, sim, orc, n)


@pytest.mark.gpu
def test_final_states_csv(tmp_path):
    model = mbg.Model.from_strings(_bnd(), _cfg())
    sim = mbg.Simulation(model, n_traj=4000).run()
    prefix = str(tmp_path / "out")
    sim.write_csv(prefix, final_states=True)
    lines = open(prefix + "_final_states.csv").read().splitlines()
    F = sim.final_states()
    reached = np.nonzero(F)[0]
    assert lines[0] == f"Final States ({reached.size})"
    outs = [model.names[i] for i in model.outputs]
    assert lines[1].split("\t") == ["Proba", "State"] + outs
    assert len(lines) == 2 + reached.size
    for line, x in zip(lines[2:], reached):
        f = line.split("\t")
        assert abs(float(f[0]) - F[x]) <= 1e-6 * max(1.0, F[x])
        on = [outs[q] for q in range(len(outs)) if (x >> q) & 1]
        assert f[1] == (" -- ".join(on) if on else "<nil>")
        assert [int(b) for b in f[2:]] == [(x >> q) & 1 for q in range(len(outs))]


@pytest.mark.gpu
def test_cli_mutants_overrides_and_final_states(tmp_path):
    (tmp_path / "m.bnd").write_text(_bnd())
    (tmp_path / "m.cfg").write_text(_cfg())
    env = dict(os.environ, MBG_MUTANTS="B:ON,C:OFF", MBG_CONFIG_EXPR="$ka = 2; sample_count = 3000;",
               MBG_FINAL_STATES_CSV="1")
    prefix = str(tmp_path / "cli")
    r = subprocess.run([mbg.CLI_PATH, "-o", prefix, str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg")],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    model = mbg.Model.from_files(str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg"),
                                 overrides="$ka = 2; sample_count = 3000;").with_mutations({"B": "ON", "C": "OFF"})
    sim = mbg.Simulation(model).run()
    lib_prefix = str(tmp_path / "lib")
    sim.write_csv(lib_prefix, final_states=True)
    for suffix in ("_probtraj.csv", "_fp.csv", "_final_states.csv"):
        assert open(prefix + suffix).read() == open(lib_prefix + suffix).read(), suffix


def test_cli_rejects_bad_mutant_and_override_specs(tmp_path):
    """Both are read before any device work: an unknown node or value, or an override that does not
    parse, ends the run with status 1 and a message."""
    (tmp_path / "m.bnd").write_text(_bnd())
    (tmp_path / "m.cfg").write_text(_cfg())
    args = [mbg.CLI_PATH, str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg")]
    for env, text in (({"MBG_MUTANTS": "Q:ON"}, "MBG_MUTANTS"), ({"MBG_MUTANTS": "A:UP"}, "MBG_MUTANTS"),
                      ({"MBG_CONFIG_EXPR": "$ka = ;"}, "<overrides>")):
        r = subprocess.run(args, capture_output=True, text=True, env=dict(os.environ, **env), timeout=600)
        assert r.returncode == 1 and text in r.stderr, (env, r.stderr)
