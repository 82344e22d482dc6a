"""Batched sweeps (mbg_batch_*): every instance of one graph-captured launch gives exactly what
its own single simulation gives — same trajectories (keyed by seed and id), same integer
arithmetic — whatever the launch shape."""
import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import golden_model

pytestmark = pytest.mark.gpu


def instances():
    texts = []
    for i in range(6):
        net = synth.sweep_instance(i)
        texts.append((net.bnd(), net.cfg(sample_count=min(net.sample_count, 3000))))
    texts.append(golden_model("montagud"))
    texts.append(golden_model("cellcycle"))
    return texts


def single(bnd, cfg, n, seed):
    m = mbg.Model.from_strings(bnd, cfg)
    s = mbg.Simulation(m, n_traj=n, seed=seed, layout=mbg.LAYOUT_WARP).run()
    return s


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
        check_same(batch, i, single(b, c, n[i], seeds[i]))


@pytest.mark.parametrize("block", [64, 256])
def test_batch_shape_does_not_change_results(block):
    texts = instances()[:4]
    models = [mbg.Model.from_strings(b, c) for b, c in texts]
    ref = mbg.Batch(models, n_traj=[1500] * 4).run()
    other = mbg.Batch(models, n_traj=[1500] * 4, block_size=block).run()
    for i in range(4):
        assert np.array_equal(ref.probtraj_raw(i)[0], other.probtraj_raw(i)[0])
        assert np.array_equal(ref.final_states(i), other.final_states(i))


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
    shape = batch.shape()
    assert shape["block_size"] in (64, 128, 256) and shape["grid"] > 0


def test_batch_probabilities_are_normalised():
    net = synth.sweep_instance(1)
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    batch = mbg.Batch([m, m], n_traj=[4000, 6000], seeds=[1, 2]).run()
    for i in range(2):
        P, _ = batch.probtraj(i)
        assert np.allclose(P.sum(axis=1), 1.0, atol=1e-6)
        assert abs(batch.final_states(i).sum() - 1.0) < 1e-12
