"""The screening logic of upmabossg_gb300.screen on the CPU, with a scripted surrogate and simulator:
which candidates are reported (predicted P(target) >= threshold, likeliest first, at most
max_report), which are re-simulated (the reported ones and every one whose ensemble spread exceeds
the cut, each once), and the TV error of the reported points against their re-simulations."""
import numpy as np

from upmabossg_gb300 import screen

S = 4  # output states


def candidates(n):
    # column 0 carries the candidate's index (log10 of it after encoding); the rest are filler scales
    c = np.ones((n, 3))
    c[:, 0] = np.arange(1, n + 1)
    return c


def index_of(encoded):
    return np.rint(10.0 ** encoded[:, 0].astype(np.float64)).astype(int) - 1


class ScriptedSurrogate:
    """Predicts from tables indexed by candidate: P(target) score, spread, full distribution."""

    out_dim = S

    def __init__(self, score, spread, dist):
        self.score, self.spread, self.dist = score, spread, dist

    def predict_column(self, x, target):
        i = index_of(x)
        return self.score[i], self.spread[i]

    def predict(self, x):
        i = index_of(x)
        return self.dist[i], self.spread[i]


class ScriptedSim:
    """Returns each candidate's true distribution and records which candidates it was asked for."""

    def __init__(self, truth):
        self.truth = truth
        self.asked = []

    def final_window(self, scales, ids=None):
        self.asked.append(np.asarray(ids).copy())
        return self.truth[np.asarray(ids)]


def scenario(n=50, seed=0):
    rng = np.random.default_rng(seed)
    score = rng.uniform(0, 1, n)
    spread = rng.uniform(0, 0.1, n)
    dist = rng.dirichlet(np.ones(S), size=n)
    truth = np.clip(dist + rng.normal(0, 0.01, dist.shape), 0, None)
    truth /= truth.sum(axis=1, keepdims=True)
    return score, spread, dist, truth


def test_reported_and_resimulated_sets():
    score, spread, dist, truth = scenario()
    sur, sim = ScriptedSurrogate(score, spread, dist), ScriptedSim(truth)
    rep = screen.screen(sur, sim, candidates(50), target_state=2, threshold=0.7, spread_cut=0.08,
                        plain_points_per_s=100.0, max_report=1000)
    hits = np.nonzero(score >= 0.7)[0]
    assert sorted(rep.hits.tolist()) == hits.tolist()
    assert np.all(np.diff(score[rep.hits]) <= 0), "the likeliest first"
    uncertain = np.nonzero(spread > 0.08)[0]
    assert rep.uncertain == len(uncertain)
    # one simulation call, each candidate once: the reported ones and the uncertain ones
    assert len(sim.asked) == 1
    assert sim.asked[0].tolist() == np.union1d(hits, uncertain).tolist()
    assert rep.resimulated == len(np.union1d(hits, uncertain))
    tv = screen.total_variation(dist[rep.hits], truth[rep.hits])
    assert np.isclose(rep.tv_mean, tv.mean()) and np.isclose(rep.tv_max, tv.max())
    assert np.array_equal(rep.hit_probs, dist[rep.hits]) and np.array_equal(rep.hit_truth, truth[rep.hits])
    assert np.isclose(rep.speedup, rep.screened_points_per_s / 100.0)


def test_report_cap_keeps_the_likeliest():
    score, spread, dist, truth = scenario(seed=1)
    sur, sim = ScriptedSurrogate(score, spread, dist), ScriptedSim(truth)
    rep = screen.screen(sur, sim, candidates(50), target_state=0, threshold=0.2, spread_cut=1.0,
                        plain_points_per_s=100.0, max_report=5)
    assert rep.reported == 5 and rep.uncertain == 0
    assert rep.hits.tolist() == np.argsort(-score)[:5].tolist()  # the five likeliest, likeliest first
    assert sim.asked[0].tolist() == sorted(rep.hits.tolist())


def test_nothing_reported_nothing_uncertain():
    score, spread, dist, truth = scenario(seed=2)
    sur, sim = ScriptedSurrogate(np.zeros(50), np.zeros(50), dist), ScriptedSim(truth)
    rep = screen.screen(sur, sim, candidates(50), target_state=1, threshold=0.5, spread_cut=0.5,
                        plain_points_per_s=100.0)
    assert rep.reported == 0 and rep.resimulated == 0 and sim.asked == []
    assert rep.tv_mean == 0.0 and rep.tv_frac_ok == 1.0


def test_encode_and_total_variation():
    x = np.array([[0.1, 1.0, 10.0]])
    assert np.allclose(screen.encode(x), [[-1.0, 0.0, 1.0]], atol=1e-6)
    assert screen.encode(x).dtype == np.float32
    p = np.array([[0.5, 0.5, 0, 0], [1, 0, 0, 0]])
    q = np.array([[0.5, 0, 0.5, 0], [1, 0, 0, 0]])
    assert np.allclose(screen.total_variation(p, q), [0.5, 0.0])
