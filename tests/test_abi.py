"""The C ABI library loads without a GPU, exports every declared symbol, and reports errors as
status codes (never exits)."""
import ctypes
import os
import re

import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "mbg.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(mbg_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol():
    lib = ctypes.CDLL(mbg.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/mbg.h but not exported"
    assert sorted(mbg.EXPORTS) == names


def test_version_and_device_count_without_gpu():
    assert b"sm_103a" in mbg.lib().mbg_version()
    assert mbg.device_count() >= 0


def test_parse_error_is_a_status():
    with pytest.raises(mbg.MbgError) as e:
        mbg.Model.from_strings("Node A { logic = A; rate_up = 1; }", "")
    assert e.value.status == 3 and "rate_down" in e.value.message


def test_syntax_error_location():
    with pytest.raises(mbg.MbgError) as e:
        mbg.Model.from_strings("Node A {\n logic = A &; rate_up = 1; rate_down = 1; }", "")
    assert e.value.status == 3 and ":2:" in e.value.message


def test_unknown_node_in_cfg():
    with pytest.raises(mbg.MbgError) as e:
        mbg.Model.from_strings("Node A { rate_up = 1; rate_down = 1; }", "B.istate = 1;")
    assert "Unknown node B" in e.value.message


def test_missing_file_is_io_error():
    with pytest.raises(mbg.MbgError) as e:
        mbg.Model.from_files("/nonexistent.bnd", "/nonexistent.cfg")
    assert e.value.status == 2


def test_jit_compiles_without_gpu():
    net = synth.small()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    assert m.jit_check() >= 0.0


def test_sim_create_without_gpu_fails_cleanly(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    net = synth.small()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    with pytest.raises(mbg.MbgError) as e:
        mbg.Simulation(m, n_traj=10)
    assert e.value.status == 5


def test_results_before_run_is_state_error(has_gpu):
    if not has_gpu:
        pytest.skip("needs a device to create a simulation")
    net = synth.small()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    s = mbg.Simulation(m, n_traj=10)
    with pytest.raises(mbg.MbgError) as e:
        s.final_states()
    assert e.value.status == 9


def test_model_info_of_workloads():
    for name, n, outs in (("small", 20, 20), ("medium", 1000, 10)):
        net = getattr(synth, name)()
        m = mbg.Model.from_strings(net.bnd(), net.cfg())
        assert m.info.nodes == n and m.info.outputs == outs
        assert m.outputs == net.outputs
        assert m.names == net.names
        assert m.info.sample_count == net.sample_count
        assert 8 <= m.info.frac_bits <= 40


def test_trajectory_limit_is_checked_before_any_device_work(has_gpu):
    """A run holds at most 2^30 trajectories: the fixed-point hash table has twice as many slots
    as trajectories, counted in 32 bits. One more is refused as an argument error before any
    device call; exactly 2^30 passes the check (without a GPU it then fails on the device)."""
    net = synth.small()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    with pytest.raises(mbg.MbgError) as e:
        mbg.Simulation(m, n_traj=(1 << 30) + 1)
    assert e.value.status == 1 and "2^30" in e.value.message
    with pytest.raises(mbg.MbgError) as e:
        mbg.Batch([m], n_traj=[(1 << 30) + 1])
    assert e.value.status == 1 and "2^30" in e.value.message
    if not has_gpu:
        with pytest.raises(mbg.MbgError) as e:
            mbg.Simulation(m, n_traj=1 << 30)
        assert e.value.status == 5


def test_option_checks_come_before_any_device_work():
    """Out-of-range options are argument errors whether or not a GPU is present: they are checked
    before the library touches a device."""
    net = synth.small()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    for kw in (dict(lane_update=3), dict(layout=9), dict(block_size=48),
               dict(layout=mbg.LAYOUT_LANE, redraw_period=99)):
        with pytest.raises(mbg.MbgError) as e:
            mbg.Simulation(m, n_traj=100, **kw)
        assert e.value.status == 1, kw
    with pytest.raises(mbg.MbgError) as e:
        mbg.Batch([m], n_traj=[100], lane_variant=3)
    assert e.value.status == 1 and "lane_variant" in e.value.message
