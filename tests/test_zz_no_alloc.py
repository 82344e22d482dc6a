"""mbg_fixed_points_aggregate_noalloc: the fixed-point aggregation for callers that may not
allocate device memory (their host owns every allocation, or cudaMalloc could stall a
latency-critical loop). It must give exactly what the allocating path of mbg_sim_run reports
through mbg_sim_fixed_points, on every call: the scratch table is shared and reused.

This file is collected last so that a failure here comes after every other test has run."""
import ctypes

import numpy as np
import pytest

import upmabossg_gb300 as mbg

from helpers import golden_model, run_device

LIMIT = 32768


def test_rejects_more_states_than_the_limit():
    n = ctypes.c_uint32()
    st = mbg.lib().mbg_fixed_points_aggregate_noalloc(None, LIMIT + 1, 4, None, None, ctypes.byref(n), None)
    assert st == 1
    assert b"32768" in mbg.lib().mbg_last_error()


@pytest.mark.gpu
def test_noalloc_matches_allocating_path_twice():
    torch = pytest.importorskip("torch")
    # Montagud's prostate model ends mostly in fixed points, many of them distinct
    bnd, cfg = golden_model("montagud")
    n_traj = 4000
    model, sim = run_device(bnd, cfg, n_traj)
    words = model.info.words
    states, _, _, status = sim.trajectories()
    fixed = np.ascontiguousarray(states[status == 2])
    assert 0 < len(fixed) <= LIMIT
    ref_states, ref_probs = sim.fixed_points()
    expected = {tuple(int(x) for x in s): int(round(p * n_traj)) for s, p in zip(ref_states, ref_probs)}
    assert sum(expected.values()) == len(fixed)

    dev = torch.device("cuda:0")
    d_states = torch.from_numpy(fixed.view(np.int32)).to(dev)
    d_unique = torch.full_like(d_states, -1)
    d_counts = torch.zeros(len(fixed), dtype=torch.int32, device=dev)
    d_n = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        st = mbg.lib().mbg_fixed_points_aggregate_noalloc(
            ctypes.c_void_p(d_states.data_ptr()), len(fixed), words, ctypes.c_void_p(d_unique.data_ptr()),
            ctypes.c_void_p(d_counts.data_ptr()), ctypes.c_void_p(d_n.data_ptr()), ctypes.c_void_p(stream))
        assert st == 0, mbg.lib().mbg_last_error()
        torch.cuda.synchronize(dev)
        nu = int(d_n.item())
        uniq = d_unique[:nu].cpu().numpy().view(np.uint32)
        cnts = d_counts[:nu].cpu().numpy()
        got = {tuple(int(x) for x in s): int(c) for s, c in zip(uniq, cnts)}
        assert nu == len(expected), f"call {call}: {nu} distinct states, expected {len(expected)}"
        assert got == expected, f"call {call}: fixed-point counts differ from mbg_sim_fixed_points"
