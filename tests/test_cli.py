"""The MaBoSSG command line: the reference's argument rules (src/main.cpp:101-152) and output
formats (window_average_small.cpp:181-250, fixed_states.cu:154-187, the stdout report)."""
import os
import subprocess

import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import GOLDEN


def cli(*args, env=None):
    return subprocess.run([mbg.CLI_PATH, *args], capture_output=True, text=True, env=env, timeout=600)


def model_paths(name):
    return os.path.join(GOLDEN, "models", name + ".bnd"), os.path.join(GOLDEN, "models", name + ".cfg")


@pytest.mark.parametrize("args", [[], ["a.bnd"], ["-x", "p", "a.bnd", "a.cfg"], ["a", "b", "c"]])
def test_usage_line_on_wrong_arguments(args):
    r = cli(*args)
    assert r.returncode == 1
    assert r.stdout.strip() == "Usage: MaBoSSG [-o prefix] bnd_file cfg_file"


def test_missing_file_fails():
    r = cli("/nonexistent.bnd", "/nonexistent.cfg")
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_parse_error_fails(tmp_path):
    (tmp_path / "m.bnd").write_text("Node A { logic = A & ; rate_up = 1; rate_down = 1; }")
    (tmp_path / "m.cfg").write_text("")
    r = cli(str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg"))
    assert r.returncode == 1 and "syntax error" in r.stderr


def test_more_than_20_outputs_is_refused(tmp_path):
    net = synth.small()  # 20 outputs: allowed; add one more node
    bnd = net.bnd() + "Node X { logic = X; rate_up = @logic ? 1 : 0; rate_down = @logic ? 0 : 1; }\n"
    (tmp_path / "m.bnd").write_text(bnd)
    (tmp_path / "m.cfg").write_text(net.cfg())
    r = cli(str(tmp_path / "m.bnd"), str(tmp_path / "m.cfg"))
    assert r.returncode == 1
    assert "maximum of 20 non-internal nodes" in r.stderr


@pytest.mark.gpu
def test_csv_outputs(tmp_path):
    bnd, cfg = model_paths("sizek")
    small_cfg = tmp_path / "s.cfg"
    small_cfg.write_text(open(cfg).read() + "\nsample_count = 20000;\n")
    prefix = str(tmp_path / "out")
    r = cli("-o", prefix, bnd, str(small_cfg))
    assert r.returncode == 0, r.stderr
    lines = open(prefix + "_probtraj.csv").read().splitlines()
    head = lines[0].split("\t")
    assert head[:5] == ["Time", "TH", "ErrorTH", "H", "HD=0"]
    assert (len(head) - 5) % 3 == 0 and head[5:8] == ["State", "Proba", "ErrorProba"]
    assert len(lines) == 1 + 20  # sizek: max_time 100, tick 5
    model = mbg.Model.from_files(bnd, str(small_cfg))
    names = set(model.names)
    for i, line in enumerate(lines[1:]):
        f = line.split("\t")
        assert float(f[0]) == pytest.approx(5.0 * i)
        assert f[2] == "0" and f[4] == "0"
        states = f[5::3]
        probs = [float(p) for p in f[6::3]]
        assert all(e == "0" for e in f[7::3])
        assert abs(sum(probs) - 1.0) < 1e-4
        for s in states:
            assert s == "<nil>" or all(n in names for n in s.split(" -- "))
    fp = open(prefix + "_fp.csv").read().splitlines()
    assert fp[0].startswith("Fixed Points (")
    n_fp = int(fp[0][len("Fixed Points ("):-1])
    assert fp[1].split("\t") == ["FP", "Proba", "State"] + model.names
    assert len(fp) == 2 + n_fp
    for row in fp[2:]:
        f = row.split("\t")
        assert f[0].startswith("#") and len(f) == 3 + len(model.names)
        on = [n for n, b in zip(model.names, f[3:]) if b == "1"]
        assert (" -- ".join(on) or "<nil>") == f[2]


@pytest.mark.gpu
def test_stdout_report_matches_library_results():
    bnd, cfg = model_paths("cellcycle")
    r = cli(bnd, cfg)
    assert r.returncode == 0, r.stderr
    out = r.stdout.splitlines()
    assert out[0] == "final points:"
    i_fixed = out.index("fixed points:")
    windows = [l for l in out if l.startswith("window (")]
    assert len(windows) == 25 and windows[0] == "window (0, 0.2]"
    # the same run through the library: the first window is all CycD (cellcycle.cfg istate)
    model = mbg.Model.from_files(bnd, cfg)
    sim = mbg.Simulation(model).run()
    P, TH = sim.probtraj()
    final = sim.final_states()
    reported = {}
    for line in out[1:i_fixed]:
        p, s = line.split(" ", 1)
        reported[s] = float(p)
    for idx, p in enumerate(final):
        if p > 0:
            key = " -- ".join(model.names[o] for q, o in enumerate(model.outputs) if (idx >> q) & 1) or "<nil>"
            assert reported[key] == pytest.approx(p, rel=1e-5)
    w0 = out.index("window (0, 0.2]")
    assert out[w0 + 1] == "entropy: 0" and out[w0 + 3] == "1 CycD"
    assert np.allclose(P.sum(axis=1), 1.0)
