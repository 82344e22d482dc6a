"""Simulation and batch handles take their device blocks from a process-wide cache
(csrc/host/devmem.cpp): a block comes back with whatever the previous handle left in it, so every
result must still be the same as in a fresh process. A run is repeated after runs of other models
with the same buffer shapes (and the window hash table, the global-row lane layout and the batch
engine in between), and must give the same results bit for bit; so is a batch after other
batches."""
import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

pytestmark = pytest.mark.gpu


def results(sim):
    bins, sums, _ = sim.probtraj_sparse()
    fs, fp = sim.fixed_points()
    return (bins.copy(), sums.copy(), sim.tr_entropy().copy(), sim.final_states().copy(), fs.copy(), fp.copy(),
            sim.summary()["transitions"])


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a[:6], b[:6])) and a[6] == b[6]


@pytest.mark.parametrize("layout", [mbg.LAYOUT_LANE, mbg.LAYOUT_WARP, mbg.LAYOUT_LANE_GLOBAL])
def test_repeat_after_other_models(layout):
    a_net, b_net = synth.sweep_instance(3), synth.sweep_instance(4)
    a = mbg.Model.from_strings(a_net.bnd(), a_net.cfg())
    b = mbg.Model.from_strings(b_net.bnd(), b_net.cfg())
    first = results(mbg.Simulation(a, n_traj=4000, seed=5, layout=layout).run())
    # other models with the same trajectory count (same fixed-point buffer shapes), other layouts
    # and the hash window table, created and destroyed in between
    for lay in (mbg.LAYOUT_WARP, mbg.LAYOUT_LANE, mbg.LAYOUT_LANE_GLOBAL):
        s = mbg.Simulation(b, n_traj=4000, seed=6, layout=lay).run()
        results(s)
        s.close()
    s = mbg.Simulation(b, n_traj=4000, seed=7, window_table=2, window_hash_bits=10).run()
    results(s)
    s.close()
    mbg.Batch([a, b], n_traj=[4000, 4000], seeds=[8, 9]).run()
    again = results(mbg.Simulation(a, n_traj=4000, seed=5, layout=layout).run())
    assert same(first, again)


def batch_results(batch, n):
    out = []
    for i in range(n):
        raw, th = batch.probtraj_raw(i)
        fs, fp = batch.fixed_points(i)
        out.append((raw.copy(), th.copy(), batch.final_states(i).copy(), fs.copy(), fp.copy(),
                    batch.summary(i)["transitions"]))
    return out


def test_batch_repeat_after_other_batches():
    """Batches take their arenas, rows and counters from the same cache: a batch repeated after
    other batches of the same shapes (whose blocks it then reuses) gives the same results."""
    nets = [synth.sweep_instance(i) for i in (1, 3, 5)]
    models = [mbg.Model.from_strings(n.bnd(), n.cfg()) for n in nets]
    b = mbg.Batch(models, n_traj=[3000] * 3, seeds=[1, 2, 3]).run()
    first = batch_results(b, 3)
    b.close()
    for seeds in ([4, 5, 6], [7, 8, 9]):
        o = mbg.Batch(models[::-1], n_traj=[3000] * 3, seeds=seeds).run()
        batch_results(o, 3)
        o.close()
    b = mbg.Batch(models, n_traj=[3000] * 3, seeds=[1, 2, 3]).run()
    again = batch_results(b, 3)
    for x, y in zip(first, again):
        assert all(np.array_equal(u, v) for u, v in zip(x[:5], y[:5])) and x[5] == y[5]
