"""Surrogate-screened parameter sweeps.

A sweep point is a vector of rate-block scale factors applied to one base network; its simulated
outcome is the output-state distribution of the final window. The plain method simulates every
point with the batch engine. The screened method trains an ensemble of MLPs (mbg_surrogate_*) on
simulated points, predicts every candidate, reports the candidates that meet the screening
criterion, and re-simulates every reported point plus every point whose ensemble spread exceeds
a threshold; the simulator has the last word on every reported point, and the total-variation error
of the surrogate against those re-simulations is reported.
"""
from __future__ import annotations

import dataclasses
import math
import time

import numpy as np

import upmabossg_gb300 as mbg


def encode(scales: np.ndarray) -> np.ndarray:
    """Network input: log10 of the scales, in [-1, 1] for scales in [0.1, 10], computed in float32
    (within 6e-8 of the float64 logarithm, far below the network's BF16 inputs; 40% less time on
    a million candidates)."""
    return np.log10(np.asarray(scales, dtype=np.float32))


def total_variation(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    return 0.5 * np.abs(np.asarray(p, np.float64) - np.asarray(q, np.float64)).sum(axis=-1)


@dataclasses.dataclass
class SimStats:
    points: int = 0
    seconds: float = 0.0        # wall time of the simulation calls
    device_ms: float = 0.0      # device time of the batched launches
    transitions: int = 0


class PointSimulator:
    """Simulates sweep points of a base model with the batch engine, chunk by chunk."""

    def __init__(self, base: mbg.Model, blocks: np.ndarray, n_traj: int, chunk: int = 1024, seed: int = 1):
        self.base = base
        self.blocks = np.asarray(blocks)
        self.n_traj = int(n_traj)
        self.chunk = int(chunk)
        self.seed = int(seed)
        self.stats = SimStats()

    def final_window(self, scales: np.ndarray, ids: np.ndarray | None = None) -> np.ndarray:
        """Final-window output-state distributions (points x 2^outputs). Point ids key the seeds, so
        a point simulated twice gives the same distribution."""
        scales = np.asarray(scales, dtype=np.float64)
        ids = np.arange(len(scales)) if ids is None else np.asarray(ids)
        out = np.zeros((len(scales), 1 << self.base.info.outputs), np.float64)
        t0 = time.perf_counter()
        for c0 in range(0, len(scales), self.chunk):
            sl = slice(c0, min(len(scales), c0 + self.chunk))
            models = []
            for s in scales[sl]:
                f = s[self.blocks]
                models.append(self.base.with_rate_scales(f, f))
            seeds = [self.seed * 1_000_003 + int(i) for i in ids[sl]]
            batch = mbg.Batch(models, n_traj=[self.n_traj] * len(models), seeds=seeds).run()
            s = batch.summary()
            self.stats.device_ms += s["sim_ms"]
            self.stats.transitions += s["transitions"]
            out[sl] = batch.window_probs(-1)
            batch.close()
            for m in models:
                m.close()
        self.stats.points += len(scales)
        self.stats.seconds += time.perf_counter() - t0
        return out


@dataclasses.dataclass
class ScreenReport:
    candidates: int
    reported: int
    uncertain: int
    resimulated: int
    predict_s: float
    resim_s: float
    tv_mean: float
    tv_max: float
    tv_frac_ok: float           # share of re-simulated reported points with TV <= 0.01
    plain_points_per_s: float
    screened_points_per_s: float
    speedup: float
    hits: np.ndarray = None          # indices of the reported candidates
    hit_probs: np.ndarray = None     # their predicted distributions
    hit_truth: np.ndarray = None     # their re-simulated distributions


def screen(surrogate: mbg.Surrogate, sim: PointSimulator, candidates: np.ndarray, target_state: int,
           threshold: float, spread_cut: float, plain_points_per_s: float, max_report: int = 1000) -> ScreenReport:
    """Reports candidates whose predicted P(target_state) >= threshold (at most max_report, the most
    likely first) and re-simulates them together with every candidate whose ensemble spread
    exceeds spread_cut."""
    t0 = time.perf_counter()
    # the target state's probability and the spread for every candidate; full distributions only
    # for the reported ones
    score, spread = surrogate.predict_column(encode(candidates), target_state)
    hits = np.nonzero(score >= threshold)[0]
    hits = hits[np.argsort(-score[hits])][:max_report]
    hit_probs = surrogate.predict(encode(candidates[hits]))[0] if len(hits) else np.zeros((0, surrogate.out_dim))
    predict_s = time.perf_counter() - t0
    uncertain = np.nonzero(spread > spread_cut)[0]
    todo = np.union1d(hits, uncertain)
    t1 = time.perf_counter()
    truth = sim.final_window(candidates[todo], ids=todo) if len(todo) else np.zeros((0, hit_probs.shape[1]))
    resim_s = time.perf_counter() - t1
    pos = {int(i): k for k, i in enumerate(todo)}
    tv = np.array([total_variation(hit_probs[k], truth[pos[int(i)]]) for k, i in enumerate(hits)]) \
        if len(hits) else np.zeros(0)
    total_s = predict_s + resim_s
    screened = len(candidates) / total_s if total_s > 0 else math.inf
    return ScreenReport(
        candidates=len(candidates), reported=len(hits), uncertain=len(uncertain), resimulated=len(todo),
        predict_s=predict_s, resim_s=resim_s, tv_mean=float(tv.mean()) if len(tv) else 0.0,
        tv_max=float(tv.max()) if len(tv) else 0.0, tv_frac_ok=float((tv <= 0.01).mean()) if len(tv) else 1.0,
        plain_points_per_s=plain_points_per_s, screened_points_per_s=screened,
        speedup=screened / plain_points_per_s if plain_points_per_s > 0 else math.inf,
        hits=hits, hit_probs=hit_probs,
        hit_truth=np.array([truth[pos[int(i)]] for i in hits]) if len(hits) else np.zeros((0, hit_probs.shape[1])))
