"""Surrogate MLP on the GPU (mbg_surrogate_*) against the CPU reference oracle/mlp.py, and what
a trained surrogate gains on a small screening sweep."""
import time

import numpy as np
import pytest

import upmabossg_gb300 as mbg
from oracle import mlp

pytestmark = pytest.mark.gpu

DIMS = [32, 512, 512, 512, 256]


def make(ensemble=1, seed=5):
    return mbg.Surrogate(32, 256, hidden=512, hidden_layers=3, ensemble=ensemble, seed=seed)


def data(rng, n):
    x = rng.uniform(-1, 1, size=(n, 32)).astype(np.float32)
    y = rng.dirichlet(np.full(256, 0.3), size=n).astype(np.float32)
    return x, y


def test_forward_matches_reference():
    rng = np.random.default_rng(0)
    s = make()
    p = s.params(0)
    x, _ = data(rng, 100)
    probs, spread = s.predict(x)
    z, _ = mlp.forward(p, DIMS, x)
    ref = mlp.softmax(z)
    assert np.abs(probs - ref).max() < 2e-3
    assert np.all(spread == 0.0)  # one member: no spread


@pytest.mark.parametrize("dims,rows", [((32, 512, 512, 512, 256), 300), ((24, 136, 136, 100), 129),
                                       ((32, 512, 512, 512, 256), 40000), ((24, 136, 136, 100), 40003)])
def test_tcgen05_forward_matches_mma_sync(dims, rows):
    """The tcgen05 GEMM (TMEM accumulator) and the mma.sync GEMM compute the same BF16 products with
    FP32 accumulation; only the summation order differs. Odd sizes exercise the partial tiles (rows
    and columns outside M and N, K not a multiple of the 16-wide MMA step); 40 000 rows make
    hundreds of 128 x 256 tiles, which run on the persistent kernel with two accumulators."""
    rng = np.random.default_rng(3)
    s = mbg.Surrogate(dims[0], dims[-1], hidden=dims[1], hidden_layers=len(dims) - 2, ensemble=1, seed=9)
    p = mlp.init_params(list(dims), rng)
    s.set_params(0, p)
    x = rng.uniform(-1, 1, size=(rows, dims[0])).astype(np.float32)
    s.set_tensor_path(True)
    a, _ = s.predict(x)
    s.set_tensor_path(False)
    b, _ = s.predict(x)
    assert np.abs(a - b).max() < 1e-4
    z, _ = mlp.forward(p, list(dims), x)
    assert np.abs(a - mlp.softmax(z)).max() < 2e-3


def test_predict_column_matches_full_prediction():
    """The screening read-back (one output column and the spread, per row) equals the full
    ensemble prediction's column bit for bit, across chunk boundaries and for any subset of rows
    (rows are independent in every product)."""
    rng = np.random.default_rng(5)
    s = mbg.Surrogate(32, 256, hidden=128, hidden_layers=2, ensemble=3, seed=4)
    x = rng.uniform(-1, 1, size=(70000, 32)).astype(np.float32)
    probs, spread = s.predict(x)
    for col in (0, 77, 255):
        score, sp = s.predict_column(x, col)
        assert np.array_equal(score, probs[:, col])
        assert np.array_equal(sp, spread)
    sub = np.array([3, 65535, 65536, 69999])
    p_sub, s_sub = s.predict(x[sub])
    assert np.array_equal(p_sub, probs[sub]) and np.array_equal(s_sub, spread[sub])
    with pytest.raises(mbg.MbgError):
        s.predict_column(x[:10], 256)


@pytest.mark.parametrize("rows", [96, 64, 1, 200])
def test_gradients_match_reference(rows):
    """Loss and gradients of every member of a 3-member ensemble (distinct parameters), computed by
    the training step's member-batched kernels, against the FP32 reference. Row counts below, at
    and across the 64-row tile, and a single row."""
    rng = np.random.default_rng(1)
    s = make(ensemble=3)
    ps = [mlp.init_params(DIMS, rng) for _ in range(3)]
    for e, p in enumerate(ps):
        s.set_params(e, p)
    x, y = data(rng, rows)
    for e, p in enumerate(ps):
        loss, g = s.gradients(e, x, y)
        ref_loss, ref_g = mlp.loss_and_grad(p, DIMS, x, y)
        assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss)
        o = 0
        for i, j in zip(DIMS[:-1], DIMS[1:]):
            for size in (i * j, j):
                a, b = g[o:o + size], ref_g[o:o + size]
                rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
                assert rel < 2e-2, f"member {e}, layer {i}x{j} block of {size}: relative gradient error {rel}"
                o += size


def test_gradients_of_odd_widths_match_reference():
    """Widths that are not multiples of 8 (no 16-byte loads) take the element-wise tile loads."""
    dims = [20, 100, 100, 90]
    rng = np.random.default_rng(6)
    s = mbg.Surrogate(dims[0], dims[-1], hidden=dims[1], hidden_layers=2, ensemble=2, seed=2)
    p = mlp.init_params(dims, rng)
    s.set_params(1, p)
    x = rng.uniform(-1, 1, size=(77, dims[0])).astype(np.float32)
    y = rng.dirichlet(np.full(dims[-1], 0.3), size=77).astype(np.float32)
    loss, g = s.gradients(1, x, y)
    ref_loss, ref_g = mlp.loss_and_grad(p, dims, x, y)
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss)
    rel = np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g)
    assert rel < 2e-2


def test_training_reduces_loss_and_ensemble_spread_is_informative():
    rng = np.random.default_rng(2)
    # a smooth target: distribution over 256 bins centred on a function of the inputs
    x = rng.uniform(-1, 1, size=(4096, 32)).astype(np.float32)
    centre = (np.tanh(x[:, :4].sum(axis=1)) * 100 + 128).astype(np.float64)
    bins = np.arange(256)[None, :]
    y = np.exp(-0.5 * ((bins - centre[:, None]) / 6.0) ** 2)
    y = (y / y.sum(axis=1, keepdims=True)).astype(np.float32)
    s = make(ensemble=3, seed=9)
    l0 = mlp.loss_and_grad(s.params(0), DIMS, x[:256], y[:256])[0]
    l1 = s.train(x, y, epochs=30, batch=256, lr=1e-3, seed=1)
    assert l1 < 0.6 * l0
    probs, spread = s.predict(x[:512])
    tv = 0.5 * np.abs(probs - y[:512]).sum(axis=1)
    assert tv.mean() < 0.35
    # far outside the training box the members disagree more
    far = rng.uniform(3, 5, size=(512, 32)).astype(np.float32)
    _, spread_far = s.predict(far)
    assert spread_far.mean() > spread.mean()


def test_screening_gain_on_a_small_sweep():
    """Trained on simulated points, the surrogate predicts held-out points far better than an
    untrained one, and screening candidates (predict, then re-simulate only what it reports or is
    unsure about) beats simulating every candidate."""
    from upmabossg_gb300 import screen, synth

    space = synth.surrogate_space()
    base = mbg.Model.from_strings(space.base.bnd(), space.base.cfg(max_time=20, time_tick=1))
    sim = screen.PointSimulator(base, space.blocks, n_traj=1000, chunk=512)
    rng = np.random.default_rng(4)
    train_s = space.sample(rng, 1200)
    y = sim.final_window(train_s).astype(np.float32)
    plain_rate = sim.stats.points / sim.stats.seconds
    held = space.sample(rng, 200)
    y_held = sim.final_window(held, ids=np.arange(10_000, 10_200))
    untrained = mbg.Surrogate(32, 256, ensemble=2, seed=3)
    p0, _ = untrained.predict(screen.encode(held))
    s = mbg.Surrogate(32, 256, ensemble=2, seed=3)
    s.train(screen.encode(train_s), y, epochs=40, batch=128, lr=1e-3)
    p1, _ = s.predict(screen.encode(held))
    tv0 = screen.total_variation(p0, y_held).mean()
    tv1 = screen.total_variation(p1, y_held).mean()
    assert tv1 < 0.5 * tv0, f"trained TV {tv1} vs untrained {tv0}"
    target = int(np.argmax(y.var(axis=0)))
    cands = space.sample(rng, 20000)
    rep = screen.screen(s, sim, cands, target, threshold=0.9, spread_cut=0.25, plain_points_per_s=plain_rate,
                        max_report=100)
    assert rep.resimulated < len(cands) / 5
    assert rep.speedup > 3.0, rep
