"""Seeded synthetic Boolean networks for the benchmark workloads, emitted as .bnd/.cfg text.

Every workload is written in the reference grammar (``Node X { logic = ...; rate_up = @logic ?
$u_X : 0; rate_down = @logic ? 0 : $d_X; }``, ``$var = value;``, ``X.is_internal = 1;``,
``X.istate = p;``) so the reference CLI and this library read identical inputs. Rates are printed
with 6 significant digits, the precision at which the reference's code generator prints them
(src/generator.cpp:103-106), so both builds see the same rate values.

Workloads (sizes as named):
  small      20 nodes, 2-3 regulators each, all rates 1, all outputs, istate 0.5,
             1e5 trajectories, max_time 100, tick 1, seed 42
  medium     1000 nodes, in-degree Poisson(2) capped at 6, 10% constant nodes, rates
             lognormal(0, 0.5), 10 outputs, istate 0.5, 1e6 trajectories, max_time 50, tick 0.5
  large      5000 nodes, power-law in-degree (exponent 2.5, 1..20), rates lognormal(0, 1),
             20 outputs, istate 0.3, 2^20 trajectories, max_time 20, tick 0.2
  sweep      instances of 50..2000 nodes (log-uniform) built like `small`, rates
             lognormal(0, 0.5), 8 outputs, 1e4..1e5 trajectories, max_time 30, tick 0.5
  surrogate  200 nodes built like `small`, 32 rate blocks scaled by log-uniform [0.1, 10],
             8 outputs, max_time 100, tick 1
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Network:
    names: list
    logic: list          # formula text per node
    up: np.ndarray       # rate_up value per node
    down: np.ndarray     # rate_down value per node
    outputs: list        # indices of non-internal nodes
    istate: np.ndarray   # activation probability per node
    sample_count: int
    max_time: float
    time_tick: float
    seed: int = 0
    discrete: bool = False

    def bnd(self) -> str:
        out = []
        for i, name in enumerate(self.names):
            out.append(
                f"Node {name} {{\n  logic = {self.logic[i]};\n"
                f"  rate_up = @logic ? $u_{name} : 0;\n  rate_down = @logic ? 0 : $d_{name};\n}}\n")
        return "".join(out)

    def cfg(self, sample_count=None, seed=None, max_time=None, time_tick=None) -> str:
        out = []
        for i, name in enumerate(self.names):
            out.append(f"$u_{name} = {fmt_rate(self.up[i])};\n$d_{name} = {fmt_rate(self.down[i])};\n")
        outs = set(self.outputs)
        for i, name in enumerate(self.names):
            if i not in outs:
                out.append(f"{name}.is_internal = 1;\n")
        for i, name in enumerate(self.names):
            out.append(f"{name}.istate = {self.istate[i]:.6g};\n")
        out.append(f"sample_count = {int(sample_count or self.sample_count)};\n")
        out.append(f"max_time = {max_time or self.max_time:g};\n")
        out.append(f"time_tick = {time_tick or self.time_tick:g};\n")
        out.append(f"discrete_time = {1 if self.discrete else 0};\n")
        out.append(f"seed_pseudorandom = {int(self.seed if seed is None else seed)};\n")
        return "".join(out)

    def with_rates(self, up, down) -> "Network":
        return dataclasses.replace(self, up=np.asarray(up, dtype=np.float64),
                                   down=np.asarray(down, dtype=np.float64))


def fmt_rate(x: float) -> str:
    return f"{float(x):.6g}"


def round_rates(x: np.ndarray) -> np.ndarray:
    """Rates as the cfg text carries them (6 significant digits)."""
    return np.array([float(fmt_rate(v)) for v in x], dtype=np.float64)


def random_formula(rng: np.random.Generator, names: list, regs) -> str:
    """Random AND/OR/NOT formula over the given regulators; every regulator appears once."""
    terms = [("!" if rng.random() < 0.5 else "") + names[r] for r in regs]
    order = list(rng.permutation(len(terms)))
    terms = [terms[i] for i in order]
    while len(terms) > 1:
        j = int(rng.integers(0, len(terms) - 1))
        op = " & " if rng.random() < 0.5 else " | "
        t = f"({terms[j]}{op}{terms[j + 1]})"
        if rng.random() < 0.2:
            t = "!" + t
        terms[j:j + 2] = [t]
    return terms[0]


def _pick_regs(rng, n, i, k):
    k = min(k, n - 1)
    others = rng.choice(n - 1, size=k, replace=False)
    return [int(r) if r < i else int(r) + 1 for r in others]


def _build(rng, n, degrees, const_frac, rate_sigma, n_out, istate, sample_count, max_time, tick, seed,
           rates_one=False):
    names = [f"N{i}" for i in range(n)]
    logic = []
    const_nodes = set()
    if const_frac > 0:
        const_nodes = set(int(x) for x in rng.choice(n, size=int(round(const_frac * n)), replace=False))
    for i in range(n):
        k = int(degrees[i])
        if i in const_nodes or k == 0:
            logic.append("TRUE" if rng.random() < 0.5 else "FALSE")
        else:
            logic.append(random_formula(rng, names, _pick_regs(rng, n, i, k)))
    if rates_one:
        up = np.ones(n)
        down = np.ones(n)
    else:
        up = round_rates(rng.lognormal(0.0, rate_sigma, size=n))
        down = round_rates(rng.lognormal(0.0, rate_sigma, size=n))
    outputs = list(range(n)) if n_out >= n else sorted(int(x) for x in rng.choice(n, size=n_out, replace=False))
    return Network(names=names, logic=logic, up=up, down=down, outputs=outputs,
                   istate=np.full(n, float(istate)), sample_count=int(sample_count),
                   max_time=float(max_time), time_tick=float(tick), seed=int(seed))


def small(seed: int = 42) -> Network:
    rng = np.random.default_rng(seed)
    n = 20
    deg = rng.integers(2, 4, size=n)
    return _build(rng, n, deg, 0.0, 0.0, n, 0.5, 100_000, 100.0, 1.0, 42, rates_one=True)


def medium(seed: int = 1000) -> Network:
    rng = np.random.default_rng(seed)
    n = 1000
    deg = np.minimum(rng.poisson(2.0, size=n), 6)
    return _build(rng, n, deg, 0.10, 0.5, 10, 0.5, 1_000_000, 50.0, 0.5, seed)


def powerlaw_degrees(rng, n, exponent=2.5, kmin=1, kmax=20):
    ks = np.arange(kmin, kmax + 1)
    p = ks.astype(np.float64) ** (-exponent)
    p /= p.sum()
    return rng.choice(ks, size=n, p=p)


def large(seed: int = 5000) -> Network:
    rng = np.random.default_rng(seed)
    n = 5000
    deg = powerlaw_degrees(rng, n)
    return _build(rng, n, deg, 0.0, 1.0, 20, 0.3, 1 << 20, 20.0, 0.2, seed)


def sweep_instance(index: int, base_seed: int = 256) -> Network:
    rng = np.random.default_rng([base_seed, index])
    n = int(round(math.exp(rng.uniform(math.log(50), math.log(2000)))))
    traj = int(round(math.exp(rng.uniform(math.log(1e4), math.log(1e5)))))
    deg = rng.integers(2, 4, size=n)
    return _build(rng, n, deg, 0.0, 0.5, 8, 0.5, traj, 30.0, 0.5, base_seed * 1000 + index)


def sweep(n_instances: int = 256, base_seed: int = 256) -> list:
    return [sweep_instance(i, base_seed) for i in range(n_instances)]


@dataclasses.dataclass
class SurrogateSpace:
    base: Network
    blocks: np.ndarray   # block id (0..31) per node

    def point(self, scales) -> Network:
        s = np.asarray(scales, dtype=np.float64)[self.blocks]
        return self.base.with_rates(round_rates(self.base.up * s), round_rates(self.base.down * s))

    def sample(self, rng: np.random.Generator, count: int) -> np.ndarray:
        """Log-uniform scaling vectors in [0.1, 10]^32."""
        return np.exp(rng.uniform(math.log(0.1), math.log(10.0), size=(count, 32)))


def surrogate_space(seed: int = 200) -> SurrogateSpace:
    rng = np.random.default_rng(seed)
    n = 200
    deg = rng.integers(2, 4, size=n)
    net = _build(rng, n, deg, 0.0, 0.0, 8, 0.5, 10_000, 100.0, 1.0, seed, rates_one=True)
    blocks = rng.integers(0, 32, size=n)
    return SurrogateSpace(base=net, blocks=blocks)


WORKLOADS = {"small": small, "medium": medium, "large": large}
