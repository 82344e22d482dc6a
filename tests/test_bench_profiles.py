"""bench.py's roofline reads its figures from the committed ncu summaries in profiles/: every kernel
the bench can report on its workloads has one, with the keys the roofline needs, and the roofline
arithmetic follows from them (CPU only)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

NEEDED = ("traffic_bytes_per_launch", "issue_slot_utilisation", "warp_instructions_per_transition",
          "threads_per_warp_instruction", "branch_uniform_pct", "l2_red_per_transition")


@pytest.mark.parametrize("kernel,workload", [("mbg_sim_lane_split", "medium"), ("mbg_sim_lane", "medium"),
                                             ("mbg_sim_lane_coop", "medium"), ("mbg_sim_thread", "small"),
                                             ("mbg_sim_lane_global", "large"), ("mbg_sim_warp", "large")])
def test_profile_has_roofline_figures(kernel, workload):
    prof = bench.profile_figures(kernel, workload)
    assert prof.get("file") == f"profiles/{kernel}_{workload}.md"
    for key in NEEDED:
        assert key in prof, (kernel, key)
    assert 0 < prof["issue_slot_utilisation"] <= 1 and 0 < prof["threads_per_warp_instruction"] <= 32


def test_warp_layout_issue_figure_on_the_1000_node_workload():
    prof = bench.profile_figures("mbg_sim_warp", "medium")
    assert prof["warp_instructions_per_transition"] == 446 and prof["issue_slot_utilisation"] > 0


def test_l2_peak_figure():
    assert bench.profile_figures("l2_atomics_probe").get("l2_red_peak_per_s", 0) > 1e10


def test_issue_roofline_arithmetic():
    prof = bench.profile_figures("mbg_sim_lane_split", "medium")
    r = bench.issue_roofline(prof, 7.2e9, {"sm_max_mhz": 2070.0}, "measured")
    peak = 152 * 4 * 2070e6
    assert r["bound"] == "issue" and abs(r["peak"] - peak / 1e9) < 1e-6
    assert abs(r["frac"] - prof["warp_instructions_per_transition"] * 7.2e9 / peak) < 1e-12
    assert abs(r["thread_frac"] - r["frac"] * prof["threads_per_warp_instruction"] / 32) < 1e-12
    assert 0 < r["frac"] <= 1 and 0 < r["l2_atomics"]["frac"] < 0.1
