"""Window sums in the hash table against the dense table, through the C ABI.

The two tables hold the same integer sums, so every comparison here is exact: the reached bins
and their sums, the transition entropy, the CSV and stdout reports. Covered: every layout that
runs on the hash table (the warp layout keeps the dense table), the discrete-time counts, a table
too small for the run (grown and re-run until it holds), the automatic choice on the 20-output
and 10-output workloads, and the sparse read-backs (window bins, final states) against the dense
ones.
"""
import os

import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import compare_histograms, golden_model, run_oracle

pytestmark = pytest.mark.gpu

DENSE, HASH = 1, 2


def simulate(bnd, cfg, n, table, bits=0, **kw):
    model = mbg.Model.from_strings(bnd, cfg)
    sim = mbg.Simulation(model, n_traj=n, window_table=table, window_hash_bits=bits, **kw).run()
    return model, sim


def same_windows(a, b, same_layout=True):
    """Integer window sums and final states agree across layouts; the transition entropy (float
    arithmetic evaluated per layout) bit for bit within one layout."""
    ba, sa, pa = a.probtraj_sparse()
    bb, sb, pb = b.probtraj_sparse()
    assert np.array_equal(ba, bb), "reached bins differ"
    assert np.array_equal(sa, sb), "bin sums differ"
    assert np.array_equal(pa, pb)
    assert np.all(np.diff(ba.astype(np.int64)) > 0), "bins not in increasing order"
    assert np.all(sa > 0)
    if same_layout:
        assert np.array_equal(a.tr_entropy(), b.tr_entropy())
    assert np.array_equal(a.final_states(), b.final_states())


HASH_LAYOUTS = [mbg.LAYOUT_THREAD, mbg.LAYOUT_LANE, "lane-split", mbg.LAYOUT_LANE_GLOBAL]


def layout_kw(layout):
    """"lane-split": the lane layout with the active-node words in global memory."""
    if layout == "lane-split":
        return {"layout": mbg.LAYOUT_LANE, "lane_update": 2}
    return {"layout": layout}


@pytest.mark.parametrize("layout", HASH_LAYOUTS)
def test_hash_table_equals_dense_table(layout):
    net = synth.small()  # 20 outputs: 2^20 states per window
    bnd, cfg = net.bnd(), net.cfg()
    _, dense = simulate(bnd, cfg, 20000, DENSE, **layout_kw(layout))
    _, hashed = simulate(bnd, cfg, 20000, HASH, **layout_kw(layout))
    assert dense.summary()["window_table"] == DENSE
    s = hashed.summary()
    assert s["window_table"] == HASH and s["window_reruns"] == 0
    assert s["window_entries"] == len(hashed.probtraj_sparse()[0])
    same_windows(dense, hashed)


@pytest.mark.parametrize("layout", HASH_LAYOUTS)
def test_full_table_grows_and_reruns(layout):
    """A 1024-slot table for a run that reaches ~10^5 bins: the first attempts overflow, the run
    repeats on tables four times larger until it holds, and the result is the dense table's."""
    net = synth.small()
    bnd, cfg = net.bnd(), net.cfg()
    _, dense = simulate(bnd, cfg, 20000, DENSE, **layout_kw(layout))
    _, hashed = simulate(bnd, cfg, 20000, HASH, bits=10, **layout_kw(layout))
    s = hashed.summary()
    assert s["window_reruns"] >= 1 and s["window_hash_bits"] > 10
    assert s["window_entries"] * 2 > (1 << 10)
    same_windows(dense, hashed)
    hashed.run()  # the next run starts on a table at most half full
    s2 = hashed.summary()
    assert s2["window_reruns"] == 0 and 2 * s2["window_entries"] <= (1 << s2["window_hash_bits"])
    same_windows(dense, hashed)


def test_warp_layout_keeps_dense_table():
    """The warp layout runs on the dense window table only: a forced hash table is refused, the
    automatic table choice keeps the dense table for it beyond the size at which other layouts
    switch, and an automatic layout under a hash table is never the warp layout."""
    net = synth.small()
    model = mbg.Model.from_strings(net.bnd(), net.cfg())
    with pytest.raises(mbg.MbgError):
        mbg.Simulation(model, n_traj=1000, layout=mbg.LAYOUT_WARP, window_table=HASH)
    bnd, cfg = wide_output_network()  # 40 x 2^24 bins: 5.4 GB dense
    model, w = simulate(bnd, cfg, 3000, 0, layout=mbg.LAYOUT_WARP)
    assert w.summary()["window_table"] == DENSE
    _, h = simulate(bnd, cfg, 3000, 0)
    assert h.summary()["window_table"] == HASH and h.summary()["layout"] != mbg.LAYOUT_WARP
    same_windows(w, h, same_layout=False)
    _, t = simulate(bnd, cfg, 3000, 0, thread_cutoff=8)  # fixed cutoff: the large-model choice
    assert t.summary()["window_table"] == HASH and t.summary()["layout"] != mbg.LAYOUT_WARP


def test_discrete_time_counts():
    bnd, cfg = golden_model("cellcycle")  # discrete_time = 1
    _, dense = simulate(bnd, cfg, 30000, DENSE)
    model, hashed = simulate(bnd, cfg, 30000, HASH, bits=10)
    assert model.info.discrete_time
    same_windows(dense, hashed)


def test_hash_table_against_oracle():
    net = synth.small()
    bnd, cfg = net.bnd(), net.cfg()
    model, sim = simulate(bnd, cfg, 4000, HASH, layout=mbg.LAYOUT_THREAD, record_trajectories=True)
    orc = run_oracle(bnd, cfg, model, 4000)
    compare_histograms(model, sim, orc, 4000)


def wide_output_network(outputs=24, windows=40):
    """A random network whose 24 output nodes make a 2^24-state output space: windows x 2^24 bins
    (40 windows: 5.4 GB as a dense table), of which a few thousand trajectories reach a sliver."""
    rng = np.random.default_rng(9)
    n = outputs + 8
    names = [f"W{i}" for i in range(n)]
    lines = []
    for i, nm in enumerate(names):
        a, b = rng.choice([x for x in names if x != nm], size=2, replace=False)
        logic = f"({a} & !{b})" if i % 2 else f"({a} | {b})"
        lines.append(f"Node {nm} {{ logic = {logic}; rate_up = @logic ? 1 : 0; rate_down = @logic ? 0 : 1; }}\n")
    cfg = "".join(f"{nm}.is_internal = {0 if i < outputs else 1};\n" for i, nm in enumerate(names))
    cfg += f"max_time = {windows * 0.5};\ntime_tick = 0.5;\nsample_count = 3000;\nseed_pseudorandom = 5;\n"
    return "".join(lines), cfg


def test_automatic_choice():
    small = synth.small()
    _, s = simulate(small.bnd(), small.cfg(), 2000, 0)  # 100 x 2^20 bins: 839 MB dense, the faster table
    assert s.summary()["window_table"] == DENSE
    bnd, cfg = wide_output_network()
    model, h = simulate(bnd, cfg, 3000, 0)  # 40 x 2^24 bins: 5.4 GB dense, beyond the 2 GiB the auto mode allows
    assert model.info.outputs == 24 and h.summary()["window_table"] == HASH
    hs = h.summary()
    _, d = simulate(bnd, cfg, 3000, DENSE, layout=hs["layout"], lane_update=hs["lane_update"],
                    block_size=hs["block_size"])
    same_windows(d, h)


def test_sparse_read_equals_dense_read():
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg()
    model, sim = simulate(bnd, cfg, 20000, DENSE)
    raw, th = sim.probtraj_raw()
    probs, _ = sim.probtraj()
    bins, sums, p = sim.probtraj_sparse()
    nz = np.flatnonzero(raw.ravel())
    assert np.array_equal(nz.astype(np.uint64), bins)
    assert np.array_equal(raw.ravel()[nz], sums)
    assert np.array_equal(probs.ravel()[nz], p)


@pytest.mark.parametrize("workload", ["medium", "small", "wide"])
def test_sparse_final_states_equal_dense(workload):
    """10 outputs (counts read whole and compacted on the host), 20 and 24 outputs (compacted on
    the device)."""
    if workload == "wide":
        bnd, cfg = wide_output_network()
    else:
        net = getattr(synth, workload)()
        bnd, cfg = net.bnd(), net.cfg()
    model, sim = simulate(bnd, cfg, 4000, 0)
    states, probs = sim.final_states_sparse()
    F = sim.final_states()
    assert F.size == 1 << model.info.outputs
    nz = np.flatnonzero(F)
    assert np.array_equal(nz.astype(np.uint64), states)
    assert np.array_equal(F[nz], probs)
    counts = np.rint(probs * 4000)
    assert np.array_equal(counts / 4000, probs) and counts.sum() == 4000


def test_reports_identical(tmp_path):
    net = synth.small()
    bnd, cfg = net.bnd(), net.cfg()
    _, dense = simulate(bnd, cfg, 5000, DENSE, layout=mbg.LAYOUT_LANE)
    _, hashed = simulate(bnd, cfg, 5000, HASH, layout=mbg.LAYOUT_LANE)
    for sim, name in ((dense, "d"), (hashed, "h")):
        sim.write_csv(str(tmp_path / name))
        sim.print_results(str(tmp_path / (name + ".txt")))
    for suffix in ("_probtraj.csv", "_fp.csv"):
        with open(tmp_path / ("d" + suffix)) as f1, open(tmp_path / ("h" + suffix)) as f2:
            assert f1.read() == f2.read()
    with open(tmp_path / "d.txt") as f1, open(tmp_path / "h.txt") as f2:
        assert f1.read() == f2.read()
