"""Batched sweeps (mbg_batch_*): every instance of one graph-captured launch gives exactly what
its own single simulation gives — same trajectories (keyed by seed and id), same integer
arithmetic — whatever the launch shape."""
import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import golden_model, mixed_network

pytestmark = pytest.mark.gpu


def instances():
    texts = []
    for i in range(6):
        net = synth.sweep_instance(i)
        texts.append((net.bnd(), net.cfg(sample_count=min(net.sample_count, 3000))))
    texts.append(golden_model("montagud"))
    texts.append(golden_model("cellcycle"))
    texts.append(mixed_network(seed=3))  # multi-valued rates and a 14-regulator node
    return texts


def single(bnd, cfg, n, seed, layout=mbg.LAYOUT_WARP, lane_update=0):
    m = mbg.Model.from_strings(bnd, cfg)
    s = mbg.Simulation(m, n_traj=n, seed=seed, layout=layout, lane_update=lane_update).run()
    return s


def single_like(batch, i, bnd, cfg, n, seed):
    """The single simulation in the layout that ran instance i: window sums agree across layouts,
    and the transition entropy (float arithmetic, evaluated per layout) agrees bit for bit within
    one layout."""
    s = batch.summary(i)
    return single(bnd, cfg, n, seed, layout=s["layout"], lane_update=s["lane_update"])


def check_same(batch, i, sim):
    a, ta = batch.probtraj_raw(i)
    b, tb = sim.probtraj_raw()
    assert np.array_equal(a, b), f"instance {i}: window sums differ"
    assert np.array_equal(ta, tb), f"instance {i}: TH sums differ"
    assert np.array_equal(batch.final_states(i), sim.final_states())
    fa, pa = batch.fixed_points(i)
    fb, pb = sim.fixed_points()
    assert np.array_equal(fa, fb) and np.array_equal(pa, pb), f"instance {i}: fixed points differ"
    assert batch.summary(i)["transitions"] == sim.summary()["transitions"]


def test_batch_matches_single_runs():
    texts = instances()
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    n = [2000] * len(models)
    seeds = [17 + i for i in range(len(models))]
    batch = mbg.Batch(models, n_traj=n, seeds=seeds).run()
    tot = batch.summary()
    assert tot["trajectories"] == sum(n) and tot["errors"] == 0
    for i, (b, c) in enumerate(texts):
        check_same(batch, i, single_like(batch, i, b, c, n[i], seeds[i]))


@pytest.mark.parametrize("layout,block", [(mbg.LAYOUT_LANE, 64), (mbg.LAYOUT_LANE, 256), (mbg.LAYOUT_WARP, 64),
                                          (mbg.LAYOUT_WARP, 256), (mbg.LAYOUT_LANE_GLOBAL, 128),
                                          (mbg.LAYOUT_LANE_GLOBAL, 256)])
def test_batch_shape_does_not_change_results(layout, block):
    texts = instances()[:4]
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    ref = mbg.Batch(models, n_traj=[1500] * 4).run()
    other = mbg.Batch(models, n_traj=[1500] * 4, block_size=block, layout=layout).run()
    name = {mbg.LAYOUT_LANE: "lane", mbg.LAYOUT_WARP: "warp", mbg.LAYOUT_LANE_GLOBAL: "lane_global"}[layout]
    assert all(k["layout"] == name and k["block_size"] == block for k in other.classes())
    for i in range(4):
        assert np.array_equal(ref.probtraj_raw(i)[0], other.probtraj_raw(i)[0])
        assert np.array_equal(ref.final_states(i), other.final_states(i))
        fa, pa = ref.fixed_points(i)
        fb, pb = other.fixed_points(i)
        assert np.array_equal(fa, fb) and np.array_equal(pa, pb)


@pytest.mark.parametrize("block", [128, 256])
def test_split_rows_variant_matches(block):
    """Lane variant 2 (active words in global memory; the `_full` kernel for the class holding
    the multi-valued-rate instance) gives the default batch's results bit for bit."""
    texts = instances()
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    ref = mbg.Batch(models, n_traj=[1200] * len(models), seeds=list(range(len(models)))).run()
    other = mbg.Batch(models, n_traj=[1200] * len(models), seeds=list(range(len(models))), layout=mbg.LAYOUT_LANE,
                      block_size=block, lane_variant=2).run()
    assert all(k["layout"] == "lane" and k["variant"] == 2 for k in other.classes())
    assert all(other.summary(i)["lane_update"] == 2 for i in range(len(models)))
    for i in range(len(models)):
        assert np.array_equal(ref.probtraj_raw(i)[0], other.probtraj_raw(i)[0])
        assert np.array_equal(ref.final_states(i), other.final_states(i))
        fa, pa = ref.fixed_points(i)
        fb, pb = other.fixed_points(i)
        assert np.array_equal(fa, fb) and np.array_equal(pa, pb)
        assert ref.summary(i)["transitions"] == other.summary(i)["transitions"]


def test_size_classes():
    """Instances are grouped by node count (<= 32, 64, ..., 4096, larger), one launch each."""
    texts = instances()
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    batch = mbg.Batch(models, n_traj=[500] * len(models)).run()
    classes = batch.classes()
    bounds = [32 << c for c in range(7)] + [1 << 30]
    sizes = sorted(m.info.nodes for m in models)
    assert sum(k["instances"] for k in classes) == len(models)
    assert sum(k["trajectories"] for k in classes) == 500 * len(models)
    expect = sorted({next(c for c, b in enumerate(bounds) if n <= b) for n in sizes})
    assert len(classes) == len(expect) >= 2
    for k, c in zip(classes, expect):
        assert k["max_nodes"] <= bounds[c] and (c == 0 or k["max_nodes"] > bounds[c - 1])
        assert k["grid"] > 0 and k["kernel_ms"] > 0


def test_graph_replay_and_autotune():
    texts = instances()[:5]
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    batch = mbg.Batch(models, n_traj=[1000] * 5, autotune=True)
    batch.run()
    first = [batch.probtraj_raw(i)[0].copy() for i in range(5)]
    s1 = batch.summary()
    batch.run()
    for i in range(5):
        assert np.array_equal(first[i], batch.probtraj_raw(i)[0])
    assert batch.summary()["transitions"] == s1["transitions"]
    for k in batch.classes():
        # the autotuner timed lane and warp shapes (and global-row lane shapes for large classes)
        # and kept the fastest
        tried = {t["layout"] for t in k["timings"]}
        assert {"lane", "warp"} <= tried <= {"lane", "warp", "lane_global"}
        assert ("lane_global" in tried) == (k["max_nodes"] > 1184)  # rows over 454 B a trajectory
        best = min(k["timings"], key=lambda t: t["kernel_ms"])
        assert (k["layout"], k["block_size"], k["variant"]) == (best["layout"], best["block_size"], best["variant"])


def test_window_gather_equals_per_instance_reads():
    """mbg_batch_window_probs: one window of every instance gathered on the device, the same
    doubles as each instance's own probtraj; instances with different output counts come back as a
    list; a window beyond an instance's last is refused."""
    texts = instances()
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    batch = mbg.Batch(models, n_traj=[1500] * len(models), seeds=list(range(len(models)))).run()
    windows = min(m.info.windows for m in models)
    for w in (0, windows // 2, -1, -2):
        got = batch.window_probs(w)
        assert isinstance(got, list) and len(got) == len(models)
        for i in range(len(models)):
            P, _ = batch.probtraj(i)
            assert np.array_equal(got[i], P[w]), (w, i)
    with pytest.raises(mbg.MbgError):
        batch.window_probs(max(m.info.windows for m in models))
    same = [mbg.Model.from_strings(*texts[1])] * 5
    b2 = mbg.Batch(same, n_traj=[800] * 5, seeds=[3, 4, 5, 6, 7]).run()
    arr = b2.window_probs(-1)
    assert arr.shape == (5, 1 << same[0].info.outputs)
    for i in range(5):
        assert np.array_equal(arr[i], b2.probtraj(i)[0][-1])


def test_warp_shapes_on_the_long_pilot():
    """The autotuner re-times its closest shapes on a pilot four times longer; with the warp layout
    forced those are warp shapes, whose per-warp shared-memory slices the long pilot's work
    description carries too. The tuned batch gives the untuned one's results."""
    net = synth.sweep_instance(2)
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    n = [160000, 160000]  # 320 000 trajectories: a long pilot beyond the 262 144 of the first one
    tuned = mbg.Batch([m, m], n_traj=n, seeds=[1, 2], layout=mbg.LAYOUT_WARP, autotune=True).run()
    k = tuned.classes()[0]
    assert k["layout"] == "warp" and len(k["timings"]) >= 2
    assert tuned.summary()["errors"] == 0
    plain = mbg.Batch([m, m], n_traj=n, seeds=[1, 2], layout=mbg.LAYOUT_WARP).run()
    for i in range(2):
        assert np.array_equal(tuned.probtraj_raw(i)[0], plain.probtraj_raw(i)[0])
        assert tuned.summary(i)["transitions"] == plain.summary(i)["transitions"]


def test_batch_probabilities_are_normalised():
    net = synth.sweep_instance(1)
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    batch = mbg.Batch([m, m], n_traj=[4000, 6000], seeds=[1, 2]).run()
    for i in range(2):
        P, _ = batch.probtraj(i)
        assert np.allclose(P.sum(axis=1), 1.0, atol=1e-6)
        assert abs(batch.final_states(i).sum() - 1.0) < 1e-12


def test_sweep_shaped_batch_against_oracle():
    """Sweep instances from 50 to ~2000 nodes (the sweep workload's range, 8 outputs, lognormal
    rates, max_time 30, tick 0.5) in one batched launch, each compared with the oracle directly:
    window sums, TH, final states and fixed points of every instance."""
    import oracle

    from helpers import TWO32
    nets = sorted((synth.sweep_instance(i) for i in range(64)), key=lambda net: len(net.names))
    picked = [nets[q] for q in (0, 16, 32, 48, 63)]  # smallest, quartiles, largest of 64
    sizes = [len(net.names) for net in picked]
    assert min(sizes) < 100 and max(sizes) > 1500
    texts = [(net.bnd(), net.cfg(sample_count=300)) for net in picked]
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    seeds = [101 + i for i in range(len(models))]
    batch = mbg.Batch(models, n_traj=[300] * len(models), seeds=seeds).run()
    for i, ((b, c), m) in enumerate(zip(texts, models)):
        orc = oracle.run(b, c, n_traj=300, seed=seeds[i], keep_trajectories=True)
        n_ties = int((orc.ties != 0).sum())
        raw, th = batch.probtraj_raw(i)
        dev = raw.astype(np.float64) / TWO32
        scale = 300 * m.info.time_tick
        tol = 1e-5 * scale + (n_ties + 1) * m.info.time_tick * 1.01
        assert np.abs(dev - orc.dense_hist()).max() <= tol, f"instance {i} ({sizes[i]} nodes): window sums"
        assert np.allclose(th / TWO32, orc.th, rtol=1e-4, atol=1e-4 * scale + n_ties * 5 * m.info.time_tick)
        fin = np.rint(batch.final_states(i) * 300)
        assert np.abs(fin - orc.final).sum() <= 2 * n_ties, f"instance {i}: final states"
        assert batch.summary(i)["transitions"] == orc.counters["transitions"] or n_ties > 0
        fs, fp = batch.fixed_points(i)
        ofix = orc.states[orc.status == 2]
        if n_ties == 0:
            assert len(fs) == (len(np.unique(ofix, axis=0)) if len(ofix) else 0), f"instance {i}: fixed points"
