"""GPU path versus the host FP64 oracle on the same Philox streams, through the C ABI.

Per trajectory: end state words, status and number of transitions bit-exact, end time within
1e-5 relative; trajectories the oracle flags as ties (an FP32 dt landing within 1e-6 of max_time,
or an FP64 pick that differs from the exact fixed-point pick) are counted and excluded.
Aggregates: window sums within 1e-5 x n x tick, TH within 1e-4 relative, final states and fixed
points exact.
"""
import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import compare_histograms, compare_trajectories, golden_model, mixed_network, run_device, run_oracle

pytestmark = pytest.mark.gpu


ALL_LAYOUTS = [mbg.LAYOUT_THREAD, mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, "lane-serial", "lane-split", mbg.LAYOUT_LANE_GLOBAL]


def layout_kw(layout):
    """Simulation keyword arguments for a layout id; "lane-serial" is the lane layout with each
    lane updating its own readers, "lane-split" the same with the active-node words in global
    memory."""
    if layout == "lane-serial":
        return {"layout": mbg.LAYOUT_LANE, "lane_update": 1}
    if layout == "lane-split":
        return {"layout": mbg.LAYOUT_LANE, "lane_update": 2}
    return {"layout": layout}


@pytest.mark.parametrize("layout", ALL_LAYOUTS)
def test_small_network_parity(layout):
    net = synth.small()
    bnd, cfg = net.bnd(), net.cfg()
    n = 4000
    model, sim = run_device(bnd, cfg, n, **layout_kw(layout))
    orc = run_oracle(bnd, cfg, model, n)
    s = sim.summary()
    assert s["layout"] == layout_kw(layout)["layout"]
    assert s["transitions"] == orc.counters["transitions"] or orc.counters["time_ties"] > 0
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, n)


@pytest.mark.parametrize("layout", ALL_LAYOUTS)
@pytest.mark.parametrize("seed,discrete", [(3, False), (4, False), (3, True)])
def test_mixed_rate_forms_parity(seed, discrete, layout):
    """Multi-valued (palette) rates reading other nodes, XOR, nested ternaries, comparisons,
    constant nodes and a 14-regulator node, in continuous and discrete time."""
    bnd, cfg = mixed_network(seed=seed, discrete=discrete)
    model, sim = run_device(bnd, cfg, 2000, **layout_kw(layout))
    assert model.info.palette_nodes > 0 and model.info.max_regulators > 12
    orc = run_oracle(bnd, cfg, model, 2000)
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, 2000)


@pytest.mark.parametrize("layout", [mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, "lane-serial", "lane-split", mbg.LAYOUT_LANE_GLOBAL])
def test_medium_network_parity(layout):
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg(sample_count=192)
    model, sim = run_device(bnd, cfg, 192, **layout_kw(layout))
    assert sim.summary()["layout"] == layout_kw(layout)["layout"]
    if "lane_update" in layout_kw(layout):
        assert sim.summary()["lane_update"] == layout_kw(layout)["lane_update"]
    orc = run_oracle(bnd, cfg, model, 192)
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, 192)


@pytest.mark.parametrize("layout", ALL_LAYOUTS)
def test_mid_network_parity(layout):
    net = synth.sweep_instance(2)  # 268 nodes, 8 outputs, lognormal rates
    bnd, cfg = net.bnd(), net.cfg(sample_count=400)
    model, sim = run_device(bnd, cfg, 400, **layout_kw(layout))
    orc = run_oracle(bnd, cfg, model, 400)
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, 400)


def wide_network(n=72, seed=5):
    """Two-valued nodes over every regulator count from 0 to 14: table and regulators in the lane
    record (k <= 4), in its 32-byte side entry with the table inline (k = 5, 6) or in the shared
    table array (k = 7..12), and in the general node records (k > 12)."""
    rng = np.random.default_rng(seed)
    names = [f"W{i}" for i in range(n)]
    lines = []
    for i, nm in enumerate(names):
        k = i % 15
        regs = list(rng.choice([x for x in names if x != nm], size=k, replace=False))
        if k == 0:
            logic = "1" if i % 2 else "0"
        else:
            logic = regs[0]
            for j, r in enumerate(regs[1:]):
                op = (" & ", " | ", " ^ ")[int(rng.integers(0, 3))]
                logic = f"({logic}{op}{'!' if j % 3 == 1 else ''}{r})"
        u = float(np.round(rng.lognormal(0.0, 0.5), 4))
        d = float(np.round(rng.lognormal(0.0, 0.5), 4))
        lines.append(f"Node {nm} {{ logic = {logic}; rate_up = @logic ? {u} : 0; rate_down = @logic ? 0 : {d}; }}\n")
    out = set(rng.choice(names, size=8, replace=False))
    cfg = "".join(f"{nm}.is_internal = {0 if nm in out else 1};\n" for nm in names)
    cfg += "max_time = 10;\ntime_tick = 0.5;\nsample_count = 3000;\nseed_pseudorandom = 17;\n"
    return "".join(lines), cfg


@pytest.mark.parametrize("layout", ALL_LAYOUTS)
def test_wide_node_parity(layout):
    bnd, cfg = wide_network()
    model, sim = run_device(bnd, cfg, 3000, **layout_kw(layout))
    assert model.info.max_regulators == 14
    orc = run_oracle(bnd, cfg, model, 3000)
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, 3000)


@pytest.mark.parametrize("layout", [mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, "lane-split", mbg.LAYOUT_LANE_GLOBAL])
def test_large_network_parity(layout):
    """The 5000-node workload at its own max_time (20) and tick (0.2): 256 trajectories of about
    7000 transitions each, every window compared."""
    net = synth.large()
    bnd, cfg = net.bnd(), net.cfg(sample_count=256)
    model, sim = run_device(bnd, cfg, 256, **layout_kw(layout))
    assert model.info.max_time == 20.0 and model.info.windows == 100
    orc = run_oracle(bnd, cfg, model, 256)
    assert orc.counters["transitions"] > 256 * 1000
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, 256)


@pytest.mark.parametrize("layout", [mbg.LAYOUT_AUTO, "lane-serial", "lane-split"])
def test_medium_network_parity_2000(layout):
    """2000 trajectories of the 1000-node workload, the autotuned kernel included."""
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg(sample_count=2000)
    model, sim = run_device(bnd, cfg, 2000, **layout_kw(layout))
    orc = run_oracle(bnd, cfg, model, 2000)
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, 2000)


@pytest.mark.parametrize("layout", [mbg.LAYOUT_AUTO, mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, "lane-serial",
                                    "lane-split", mbg.LAYOUT_LANE_GLOBAL])
@pytest.mark.parametrize("name,n", [("cellcycle", 3000), ("metastasis", 300), ("sizek", 300), ("montagud", 200)])
def test_reference_models_parity(name, n, layout):
    bnd, cfg = golden_model(name)
    model, sim = run_device(bnd, cfg, n, **layout_kw(layout))
    orc = run_oracle(bnd, cfg, model, n)
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, n)


@pytest.mark.parametrize("other", [mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, "lane-serial", "lane-split", mbg.LAYOUT_LANE_GLOBAL])
def test_layouts_agree(other):
    """Every layout runs the same integer arithmetic and the same clock: identical window sums,
    final states and fixed points."""
    net = synth.sweep_instance(2)
    bnd, cfg = net.bnd(), net.cfg(sample_count=3000)
    _, a = run_device(bnd, cfg, 3000, layout=mbg.LAYOUT_THREAD, record=False)
    _, b = run_device(bnd, cfg, 3000, record=False, **layout_kw(other))
    ra, _ = a.probtraj_raw()
    rb, _ = b.probtraj_raw()
    assert np.array_equal(ra, rb)
    assert np.array_equal(a.final_states(), b.final_states())
    fa, pa = a.fixed_points()
    fb, pb = b.fixed_points()
    assert np.array_equal(fa, fb) and np.array_equal(pa, pb)
    assert a.summary()["transitions"] == b.summary()["transitions"]


def test_run_is_deterministic():
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg(sample_count=2000)
    model, sim = run_device(bnd, cfg, 2000, record=False)
    r1, t1 = sim.probtraj_raw()
    s1 = sim.summary()
    sim.run()
    r2, t2 = sim.probtraj_raw()
    assert np.array_equal(r1, r2) and np.array_equal(t1, t2)
    assert sim.summary()["transitions"] == s1["transitions"]


def test_trajectory_ids_are_partition_independent():
    """Philox is keyed by trajectory id: two runs over [0, n/2) and [n/2, n) equal one run."""
    net = synth.small()
    bnd, cfg = net.bnd(), net.cfg()
    _, full = run_device(bnd, cfg, 1000, record=False)
    _, lo = run_device(bnd, cfg, 500, record=False)
    _, hi = run_device(bnd, cfg, 500, record=False, traj_base=500)
    a, _ = full.probtraj_raw()
    b, _ = lo.probtraj_raw()
    c, _ = hi.probtraj_raw()
    assert np.array_equal(a, b + c)


@pytest.mark.parametrize("layout", [mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, "lane-serial", "lane-split", mbg.LAYOUT_LANE_GLOBAL])
def test_step_limit_is_counted(layout):
    net = synth.medium()
    bnd, cfg = net.bnd(), net.cfg(sample_count=64)
    model, sim = run_device(bnd, cfg, 64, max_steps=50, **layout_kw(layout))
    s = sim.summary()
    assert s["step_limited"] > 0
    assert s["step_limited"] + s["finished"] + s["fixed_points"] == 64
    st, t, tr, status = sim.trajectories()
    assert np.all(tr[status == 3] == 50)
    orc = run_oracle(bnd, cfg, model, 64, max_steps=50)
    assert np.array_equal(status, orc.status)


@pytest.mark.parametrize("workload,n,layout", [("medium", 192, mbg.LAYOUT_WARP), ("mid", 1000, mbg.LAYOUT_WARP),
                                               ("mid", 1000, mbg.LAYOUT_THREAD)])
def test_reference_segment_process_parity(workload, n, layout):
    """redraw_period = 99 (the reference build's launch segments): trajectory for trajectory against
    the oracle running the same process."""
    net = synth.medium() if workload == "medium" else synth.sweep_instance(2)
    bnd, cfg = net.bnd(), net.cfg(sample_count=n)
    model, sim = run_device(bnd, cfg, n, layout=layout, redraw_period=99)
    orc = run_oracle(bnd, cfg, model, n, redraw_period=99)
    exact = run_oracle(bnd, cfg, model, n)
    assert orc.counters["steps"] > exact.counters["steps"]  # the segment ends are extra steps
    assert sim.summary()["steps"] == orc.counters["steps"] or orc.counters["time_ties"] > 0
    compare_trajectories(sim, orc)
    compare_histograms(model, sim, orc, n)


def test_reference_segment_process_needs_thread_or_warp():
    net = synth.small()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    for lay in (mbg.LAYOUT_LANE, mbg.LAYOUT_LANE_GLOBAL):
        with pytest.raises(mbg.MbgError) as e:
            mbg.Simulation(m, n_traj=100, layout=lay, redraw_period=99)
        assert e.value.status == 1
    s = mbg.Simulation(m, n_traj=1000, redraw_period=99).run()  # auto: tuned over thread and warp only
    assert s.summary()["layout"] in (mbg.LAYOUT_THREAD, mbg.LAYOUT_WARP)
