"""Benchmark: transitions/s of the GPU simulator on one GB300 (and its CPU reference arm).

Default workload: the 1000-node synthetic network (in-degree Poisson(2) capped at 6, 10% constant
nodes, lognormal(0, 0.5) rates, 10 outputs, 1e6 trajectories, max_time 50, tick 0.5), generated
from a fixed seed. One step is one full simulation of all trajectories (mbg_sim_run), including
the clearing of the result buffers and the fixed-point aggregation. The L2 is flushed (256 MiB
write) between timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload medium|small|large]
  python bench.py --impl reference ...   # the CPU restatement of the reference path

Under torchrun (WORLD_SIZE > 1) every rank simulates its own range of trajectory ids (weak
scaling); there is no collective on the data path, only a barrier and a max over ranks of the
step time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "small": "20-node random network, 2-3 regulators per node, all rates 1, all nodes output, istate 0.5, "
             "1e5 trajectories, max_time 100, tick 1, seed 42",
    "medium": "1000-node random network, in-degree Poisson(2) capped at 6, 10% constant nodes, rates "
              "lognormal(0,0.5), 10 outputs, istate 0.5, 1e6 trajectories, max_time 50, tick 0.5",
    "large": "5000-node random network, power-law in-degree (2.5, 1..20), rates lognormal(0,1), 20 outputs, "
             "istate 0.3, 2^20 trajectories, max_time 20, tick 0.2",
}
CPU_SAMPLE_SECONDS = 15.0


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


MBG_LAYOUTS = {"thread": 1, "warp": 2, "lane": 3, "lane_global": 4}


PROFILE_KEYS = ("traffic_bytes_per_launch", "issue_slot_utilisation", "warp_instructions_per_transition",
                "threads_per_warp_instruction", "branch_uniform_pct", "l2_red_per_transition", "l2_red_peak_per_s")


def profile_figures(kernel, workload=None):
    """Figures of the committed ncu summary profiles/<kernel>_<workload>.md (or profiles/<kernel>.md):
    its `key: value` lines (PROFILE_KEYS)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md" if workload else f"{kernel}.md")
    out = {}
    if not os.path.exists(path):
        return out
    out["file"] = os.path.relpath(path, ROOT)
    with open(path) as f:
        for line in f:
            key, sep, val = line.strip().strip("`").partition(": ")
            if sep and key in PROFILE_KEYS:
                try:
                    out[key] = float(val) if ("." in val or "e" in val) else int(val)
                except ValueError:
                    pass
    return out


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def model_work_per_transition(net, info):
    """Thread-level operations of one transition of the reference algorithm (every rate
    re-evaluated, summed and scanned): sum_i c_i + 2N + 4 n_out + 40, where c_i counts one
    extract per regulator reference, one op per AND/OR/NOT and 2 for the compare and select."""
    total = 0
    for f in net.logic:
        refs = sum(1 for tok in f.replace("(", " ").replace(")", " ").replace("!", " ! ").split()
                   if tok.startswith("N"))
        ops = f.count("&") + f.count("|") + f.count("!")
        total += 2 * refs + ops + 2
    return total + 2 * info.nodes + 4 * info.outputs + 40


def issue_roofline(prof, transitions_per_s, peaks, peaks_kind, sms=152):
    """Instruction-issue roofline of a simulation kernel: warp instructions per transition (from
    the committed ncu summary of the kernel on this workload) x transitions/s, against the issue
    peak of one warp instruction per scheduler per clock (sms x 4 x clock). `thread_frac` scales
    that by the threads active per warp instruction / 32 (the SIMT lanes doing useful work)."""
    clock = peaks.get("sm_max_mhz", 2070.0) * 1e6
    peak = sms * 4 * clock
    out = {"bound": "issue", "unit": "G warp-instructions/s", "peak": peak / 1e9,
           "peak_source": f"{sms} SMs x 4 schedulers x {clock / 1e6:.0f} MHz ({peaks_kind} sm_max_mhz)",
           "issue_slot_utilisation_ncu": prof.get("issue_slot_utilisation"),
           "branch_efficiency_ncu": (prof["branch_uniform_pct"] / 100.0) if "branch_uniform_pct" in prof else None}
    # the secondary bound: the window flushes' L2 reductions against the measured L2 peak
    l2 = profile_figures("l2_atomics_probe")
    if prof.get("l2_red_per_transition") and l2.get("l2_red_peak_per_s"):
        red = prof["l2_red_per_transition"] * transitions_per_s
        out["l2_atomics"] = {"achieved": red, "peak": l2["l2_red_peak_per_s"], "unit": "u64 reductions/s",
                             "frac": red / l2["l2_red_peak_per_s"], "per_transition": prof["l2_red_per_transition"],
                             "peak_source": l2.get("file")}
    wpt = prof.get("warp_instructions_per_transition")
    if wpt:
        achieved = wpt * transitions_per_s
        out.update({"achieved": achieved / 1e9, "frac": achieved / peak,
                    "warp_instructions_per_transition": wpt})
        tpw = prof.get("threads_per_warp_instruction")
        if tpw:
            out.update({"threads_per_warp_instruction": tpw, "thread_frac": achieved / peak * tpw / 32.0})
    else:
        out.update({"achieved": None, "frac": None})
    return out


def make_network(name):
    from upmabossg_gb300 import synth
    return getattr(synth, name)()


def cpu_reference(net, bnd, cfg, frac_bits, seconds, threads=0, seed=None):
    """Times the oracle port (the reference path restated on the CPU) on a bounded sample."""
    import oracle
    pilot = oracle.run(bnd, cfg, frac_bits=frac_bits, n_traj=32, threads=threads, seed=seed)
    per_traj = max(pilot.seconds / 32 * pilot.threads, 1e-6)  # thread-seconds per trajectory
    ncores = threads or (os.cpu_count() or 1)
    n = int(max(64, min(net.sample_count, seconds * ncores / per_traj)))
    r = oracle.run(bnd, cfg, frac_bits=frac_bits, n_traj=n, threads=threads, seed=seed)
    tps = r.counters["transitions"] / r.seconds
    return {"value": tps, "unit": "transitions/s", "cores": r.threads, "kind": "port",
            "sample": f"first {n} of {net.sample_count} trajectories ({r.counters['transitions']} transitions, "
                      f"{r.seconds:.1f} s)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle  # noqa: F401
    net = make_network(args.workload)  # the workload's text only: libmbg.so is never loaded here
    bnd, cfg = net.bnd(), net.cfg()
    vals, ms = [], []
    last = None
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        last = cpu_reference(net, bnd, cfg, 0, args.cpu_seconds / 2)  # 0: the oracle derives the scale
        if i >= args.warmup:
            vals.append(last["value"])
            ms.append((time.perf_counter() - t0) * 1e3)
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": "transitions/s", "value": value, "unit": "transitions/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "trajectories_per_gpu": args.n_traj or net.sample_count,
                       "step": "a bounded sample of the workload's trajectories per step (see cpu_baseline.sample)"},
            "cpu_baseline": dict(last, value=value),
            "e2e": {"value": value, "unit": "transitions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


SWEEP_DESC = ("256 instances, 50..2000 nodes (log-uniform), 2-3 regulators per node, rates lognormal(0,0.5), "
              "8 outputs, 1e4..1e5 trajectories (log-uniform), max_time 30, tick 0.5")


def sweep_models(n_instances=256):
    import upmabossg_gb300 as mbg
    from upmabossg_gb300 import synth
    nets = synth.sweep(n_instances)
    return nets, [mbg.Model.from_strings(n.bnd(), n.cfg()) for n in nets]


def measure_sweep(steps, warmup, local=0, autotune=True):
    """Plain batched simulation of the sweep: every instance simulated in one graph launch.
    Returns sweep points (instances) per second and transitions per second."""
    import upmabossg_gb300 as mbg
    nets, models = sweep_models()
    batch = mbg.Batch(models, device=local, autotune=autotune)
    for _ in range(max(1, warmup)):
        batch.run()
    ms = []
    for _ in range(steps):
        batch.run()
        ms.append(batch.summary()["sim_ms"])
    s = batch.summary()
    step_ms = statistics.mean(ms)
    return {"metric": "sweep points/s (plain batched simulation)", "value": len(models) / (step_ms * 1e-3),
            "unit": "points/s", "ms_per_step": step_ms, "transitions_per_s": s["transitions"] / (step_ms * 1e-3),
            "kernel_ms": s["kernel_ms"], "trajectories": s["trajectories"], "instances": len(models),
            "classes": batch.classes(), "workload": SWEEP_DESC}


SURROGATE_DESC = ("200-node network (2-3 regulators, rates 1) with 32 rate blocks scaled log-uniform in [0.1, 10], "
                  "8 outputs, final window of max_time 100 / tick 1; MLP 32-512-512-512-256 (BF16, FP32 accumulate), "
                  "ensemble of 4 trained 120 epochs (batch 64, Adam, cosine decay); 20000 training points x 1e4 "
                  "trajectories; 1e6 candidates")


def measure_surrogate(n_train=20000, n_traj=10000, n_cand=1_000_000, epochs=120, batch=64, seed=7, n_recall=10000,
                      with_gemm=True, label_traj=None):
    """Sweep points/s of surrogate-screened versus plain batched simulation, with the TV error of
    the surrogate against re-simulation of every reported point. Training labels are simulated
    with `label_traj` trajectories per point (default n_traj); the plain method, the held-out
    points, the recall subsample and every re-simulation use n_traj."""
    import numpy as np

    import upmabossg_gb300 as mbg
    from upmabossg_gb300 import screen, synth
    label_traj = label_traj or n_traj
    space = synth.surrogate_space()
    base = mbg.Model.from_strings(space.base.bnd(), space.base.cfg())
    sim = screen.PointSimulator(base, space.blocks, n_traj=n_traj, chunk=1024)
    label_sim = sim if label_traj == n_traj else screen.PointSimulator(base, space.blocks, n_traj=label_traj,
                                                                         chunk=1024, seed=3)
    rng = np.random.default_rng(seed)
    train = space.sample(rng, n_train)
    t0 = time.perf_counter()
    y = label_sim.final_window(train).astype(np.float32)
    data_s = time.perf_counter() - t0
    s = mbg.Surrogate(32, 256, hidden=512, hidden_layers=3, ensemble=4, seed=seed)
    t1 = time.perf_counter()
    loss = s.train(screen.encode(train), y, epochs=epochs, batch=batch, lr=1e-3, seed=seed)
    train_s = time.perf_counter() - t1
    held = space.sample(rng, 1000)
    y_held = sim.final_window(held, ids=np.arange(n_train, n_train + 1000))
    cands = space.sample(rng, n_cand)
    # the recall subsample (below) is simulated plainly here, before the screen: with the held-out
    # points it times the plain method (11 000 points at n_traj trajectories)
    sub = np.sort(rng.choice(n_cand, size=n_recall, replace=False))
    y_sub_all = sim.final_window(cands[sub], ids=sub)
    plain = sim.stats.points / sim.stats.seconds
    plain_transitions = sim.stats.transitions / sim.stats.seconds
    p_held, spread_held = s.predict(screen.encode(held))
    tv_held = screen.total_variation(p_held, y_held)
    target = int(np.argmax(y.var(axis=0)))
    # uncertainty gate: candidates whose ensemble spread exceeds the 99.9th percentile of the spread
    # over 100 000 unlabelled draws of the sweep space (in distribution by construction; a spread
    # needs no simulation) are re-simulated: about 0.1% of in-distribution candidates, and every
    # candidate the members disagree on more than on almost all in-distribution points. The 1000
    # labelled held-out points alone would put the cut at their largest spread, which moves the
    # number of re-simulated candidates several-fold between trainings.
    n_calib = 100_000
    _, spread_calib = s.predict_column(screen.encode(space.sample(rng, n_calib)), target)
    spread_cut = float(np.quantile(spread_calib, 0.999))
    hi = spread_held >= np.quantile(spread_held, 0.9)
    gate = {"spread_cut": spread_cut, "quantile": 0.999, "calibration_points": n_calib,
            "held_out_above_cut": int((spread_held > spread_cut).sum()),
            "tv_held_out_top_decile_spread": float(tv_held[hi].mean()),
            "tv_held_out_rest": float(tv_held[~hi].mean()),
            "spearman_spread_tv": float(np.corrcoef(np.argsort(np.argsort(spread_held)),
                                                    np.argsort(np.argsort(tv_held)))[0, 1])}
    threshold = 0.9
    rep = screen.screen(s, sim, cands, target, threshold=threshold, spread_cut=spread_cut, plain_points_per_s=plain,
                        max_report=1000)
    # recall of the screening criterion: a random subsample of the candidates simulated plainly;
    # a true hit has simulated P(target) >= threshold; the screen finds it when its predicted
    # P(target) >= threshold (before the report cap)
    y_sub = y_sub_all[:, target]
    score_sub, _ = s.predict_column(screen.encode(cands[sub]), target)
    true_hit = y_sub >= threshold
    found = score_sub >= threshold
    recall = {"subsample": int(n_recall), "true_hits": int(true_hit.sum()), "found": int((true_hit & found).sum()),
              "recall": float((true_hit & found).sum() / max(1, true_hit.sum())),
              "predicted_hits": int(found.sum()),
              "precision": float((true_hit & found).sum() / max(1, found.sum())),
              "true_hits_clear_of_noise": int((y_sub >= threshold + 0.02).sum()),
              "recall_clear_of_noise": float(((y_sub >= threshold + 0.02) & found).sum()
                                             / max(1, (y_sub >= threshold + 0.02).sum())),
              "criterion": f"P(target state {target}) >= {threshold} in the final window, 1e4-trajectory simulation"}
    # the re-simulations above carry sampling noise of their own (1e4 trajectories over 2^8 output
    # states); a 1e5-trajectory simulation of the same points, on independent seeds, measures the
    # surrogate's error against a 3x less noisy reference and the noise of the 1e4 runs themselves
    fine = screen.PointSimulator(base, space.blocks, n_traj=10 * n_traj, chunk=256, seed=2)
    y_fine_rep = fine.final_window(cands[rep.hits], ids=rep.hits) if len(rep.hits) else None
    y_fine_held = fine.final_window(held, ids=np.arange(n_train, n_train + 1000))

    def tv_stats(tv):
        return {"mean": float(tv.mean()), "median": float(np.median(tv)), "share_le_0.01": float((tv <= 0.01).mean()),
                "n": int(len(tv))}
    fine_ref = {"trajectories": 10 * n_traj,
                "held_out_surrogate": tv_stats(screen.total_variation(p_held, y_fine_held)),
                "held_out_1e4_simulation": tv_stats(screen.total_variation(y_held, y_fine_held))}
    if y_fine_rep is not None:
        fine_ref["reported_surrogate"] = tv_stats(screen.total_variation(rep.hit_probs, y_fine_rep))
        fine_ref["reported_1e4_simulation"] = tv_stats(screen.total_variation(rep.hit_truth, y_fine_rep))
    gemm = measure_surrogate_gemm() if with_gemm else None
    return {
        "metric": "sweep points/s, surrogate-screened vs plain batched simulation", "value": rep.screened_points_per_s,
        "unit": "points/s", "plain_points_per_s": plain, "speedup": rep.speedup,
        # the one-time cost of the surrogate (training data and training) charged to this screen
        "value_including_training": len(cands) / (data_s + train_s + rep.predict_s + rep.resim_s),
        "speedup_including_training": len(cands) / (data_s + train_s + rep.predict_s + rep.resim_s) / plain,
        "plain_transitions_per_s": plain_transitions,
        "tv_reported": {"mean": rep.tv_mean, "max": rep.tv_max, "share_le_0.01": rep.tv_frac_ok, "n": rep.reported},
        "tv_held_out": {"mean": float(tv_held.mean()), "median": float(np.median(tv_held)),
                        "share_le_0.01": float((tv_held <= 0.01).mean()), "n": len(held)},
        "resimulated": rep.resimulated, "uncertain": rep.uncertain, "candidates": rep.candidates,
        "uncertainty_gate": gate, "recall": recall,
        "predict_s": rep.predict_s, "resim_s": rep.resim_s, "train_s": train_s, "train_loss": loss,
        "training_data_s": data_s, "label_trajectories": label_traj, "tv_vs_1e5_trajectories": fine_ref, "gemm": gemm,
        "workload": SURROGATE_DESC}


def measure_surrogate_gemm(rows=131072, reps=10):
    """Tensor-core throughput of the surrogate's forward products (4 members of 32-512-512-512-256,
    BF16 in, FP32 accumulate, bias/ReLU epilogues) on the tcgen05 kernel and on the mma.sync kernel,
    against the measured cuBLAS BF16 peak."""
    import upmabossg_gb300 as mbg
    peaks, kind = load_peaks()
    dims = [32, 512, 512, 512, 256]
    flop = 2.0 * rows * 4 * sum(a * b for a, b in zip(dims[:-1], dims[1:]))
    out = {"rows": rows, "members": 4, "flop_per_pass": flop}
    for name, tc in (("tcgen05", True), ("mma_sync", False)):
        s = mbg.Surrogate(32, 256, hidden=512, hidden_layers=3, ensemble=4, seed=11, tcgen05=tc)
        ms = s.time_forward(rows, reps)
        s.close()
        tf = flop / (ms * 1e-3) / 1e12
        out[name] = {"ms_per_pass": ms, "tflops": tf, "frac_of_bf16_peak": tf / peaks["bf16_tflops"]}
    out["peak_tflops"] = peaks["bf16_tflops"]
    out["peak_source"] = f"{kind} cuBLAS bf16 burst (MEASURED_PEAKS.json)" if kind == "measured" else kind
    return out


def measure_secondary():
    """The secondary metric on the same box, compactly: sweep points/s of the plain batched engine
    on the 256-instance sweep, and surrogate-screened against plain points/s on the 1e6-candidate
    screen, with the TV error of the reported and held-out points and the screen's recall."""
    out = {"metric": "sweep points/s, surrogate-screened vs plain batched simulation, at TV <= 0.01"}
    try:
        sw = measure_sweep(2, 1)
        out["sweep"] = {k: sw[k] for k in ("value", "unit", "ms_per_step", "transitions_per_s", "instances",
                                           "trajectories")}
        out["sweep"]["workload"] = SWEEP_DESC
    except Exception as e:  # the headline line is printed whatever happens here
        out["sweep"] = {"error": repr(e)}
    try:
        su = measure_surrogate(with_gemm=False)
        keep = ("value", "unit", "plain_points_per_s", "speedup", "value_including_training",
                "speedup_including_training", "tv_reported", "tv_held_out", "uncertainty_gate", "recall",
                "resimulated", "uncertain", "candidates", "train_s", "training_data_s", "predict_s", "resim_s")
        out["surrogate"] = {k: su[k] for k in keep}
        out["surrogate"]["tv_vs_1e5_trajectories"] = su["tv_vs_1e5_trajectories"]
        out["surrogate"]["workload"] = SURROGATE_DESC
    except Exception as e:
        out["surrogate"] = {"error": repr(e)}
    return out


COLD_SCRIPT = r"""
import json, sys, time
t0 = time.perf_counter()
sys.path.insert(0, {root!r})
import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth
net = getattr(synth, {workload!r})()
bnd, cfg = net.bnd(), net.cfg()
t1 = time.perf_counter()
m = mbg.Model.from_strings(bnd, cfg)
s = mbg.Simulation(m, n_traj={n}, traj_base={base}, device={dev}, **{kw!r})
s.run()
bins, sums, probs = s.probtraj_sparse()
th = s.tr_entropy(); fst, fpr = s.final_states_sparse(); fs, fp = s.fixed_points()
t2 = time.perf_counter()
print(json.dumps({{"ms": (t2 - t1) * 1e3, "import_ms": (t1 - t0) * 1e3, "transitions": s.summary()["transitions"]}}))
"""


def e2e_cold(workload, n, base, dev, kw):
    """The end-to-end path in a new process (a command-line run): CUDA context, library load,
    kernels from the on-disk cubin cache, launch shapes from the on-disk autotune cache (both warm
    after this bench's own runs), parse, create, run and read-back."""
    code = COLD_SCRIPT.format(root=ROOT, workload=workload, n=n, base=base, dev=dev, kw=kw)
    try:
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
        d = json.loads(r.stdout.strip().splitlines()[-1])
    except Exception as e:  # reported, never fatal to the headline line
        return {"error": repr(e)}
    return {"value": d["transitions"] / (d["ms"] * 1e-3), "unit": "transitions/s", "ms": d["ms"],
            "python_import_ms": d["import_ms"],
            "path": "new process: context + parse + create (disk caches) + run + reads"}


def run_ours(args):
    ws, rank, local = dist_env()
    import upmabossg_gb300 as mbg
    if mbg.device_count() < 1:
        raise SystemExit("bench: no CUDA device")
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    net = make_network(args.workload)
    # weak scaling: every rank runs the workload's full trajectory count on its own id range
    # (trajectories are keyed by id, so the union is one run of ws x n trajectories)
    n_rank = args.n_traj or net.sample_count
    base = rank * n_rank
    bnd, cfg = net.bnd(), net.cfg()
    model = mbg.Model.from_strings(bnd, cfg)
    sim_kw = dict(layout=args.layout, block_size=args.block, lane_update=args.lane_update,
                  window_table=args.window_table)
    sim = mbg.Simulation(model, n_traj=n_rank, traj_base=base, device=local, **sim_kw)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        sim.run()
    kernel_ms, sim_ms, transitions = [], [], []
    with Clocks(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            sim.run()
            s = sim.summary()
            kernel_ms.append(s["kernel_ms"])
            sim_ms.append(s["sim_ms"])
            transitions.append(s["transitions"])
        barrier()
        wall = time.perf_counter() - t0
    step_ms = sum(sim_ms) / len(sim_ms)
    trans_step = transitions[-1]  # every step runs the same trajectories: identical counts
    if ws > 1:
        t = torch.tensor([step_ms], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(t.item())
        c = torch.tensor([trans_step], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
        trans_all = float(c.item())
    else:
        trans_all = float(trans_step)
    value = trans_all / (step_ms * 1e-3)
    summary = sim.summary()

    # end to end through the public API: parse + create (H2D of the model) + run + results (D2H)
    e2e_ms = []
    h2d = d2h = 0
    for i in range(max(2, args.steps // 2) + 1):
        t1 = time.perf_counter()
        m2 = mbg.Model.from_strings(bnd, cfg)
        s2 = mbg.Simulation(m2, n_traj=n_rank, traj_base=base, device=local, **sim_kw)
        s2.run()
        bins, sums, probs = s2.probtraj_sparse()
        TH = s2.tr_entropy()
        fst, fpr = s2.final_states_sparse()
        fs, fp = s2.fixed_points()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t1
        if i > 0:
            e2e_ms.append(dt * 1e3)
        # model text in (the model tables are built and uploaded by mbg_sim_create); out: the
        # reached window bins (u32 bin + u64 sum each), TH sums, the reached final states (u32
        # state + u32 count each), fixed points
        h2d = len(bnd) + len(cfg)
        d2h = bins.size * 12 + TH.size * 8 + fst.size * 8 + fs.nbytes + fp.size * 4
        s2.close()
        m2.close()
    e2e_step_ms = statistics.mean(e2e_ms)
    cold = e2e_cold(args.workload, n_rank, base, local, sim_kw) if rank == 0 and ws == 1 else None
    if ws > 1:
        t = torch.tensor([e2e_step_ms], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_step_ms = float(t.item())
    e2e_value = trans_all / (e2e_step_ms * 1e-3)

    peaks, peaks_kind = load_peaks()
    info = model.info
    kms = sum(kernel_ms) / len(kernel_ms)
    kernel = {MBG_LAYOUTS["thread"]: "mbg_sim_thread", MBG_LAYOUTS["warp"]: "mbg_sim_warp",
              MBG_LAYOUTS["lane"]: {0: "mbg_sim_lane_coop", 1: "mbg_sim_lane",
                                    2: "mbg_sim_lane_split"}[summary.get("lane_update", 0)],
              MBG_LAYOUTS["lane_global"]: "mbg_sim_lane_global"}[summary["layout"]]
    prof = profile_figures(kernel, args.workload)
    roofline = issue_roofline(prof, trans_step / (kms * 1e-3), peaks, peaks_kind)
    # the reference algorithm's work (every rate re-evaluated, summed and scanned per transition)
    # at this rate, against the SIMT lane peak: a work rate, not a roofline of the kernel that ran
    w_tr = model_work_per_transition(net, info)
    lane_peak = 152 * 128 * peaks.get("sm_max_mhz", 2070.0) * 1e6
    roofline.update({"kernel": kernel, "kernel_ms": kms, "traffic": prof.get("traffic_bytes_per_launch"),
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                     "profile": prof.get("file"),
                     "reference_work_rate": {
                         "ops_per_transition": w_tr, "gops": trans_step * w_tr / (kms * 1e-3) / 1e9,
                         "simt_lane_peak_gops": lane_peak / 1e9,
                         "ratio_to_lane_peak": trans_step * w_tr / (kms * 1e-3) / lane_peak}})
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_reference(net, bnd, cfg, info.frac_bits, args.cpu_seconds)
    clocks = clk.summary()
    secondary = None
    if rank == 0 and ws == 1 and not args.no_secondary and args.workload == "medium":
        sim.close()
        secondary = measure_secondary()
    line = {
        "metric": "transitions/s", "value": value, "unit": "transitions/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "trajectories_per_gpu": n_rank,
                   "transitions_per_step": trans_all,
                   "layout": ["", "thread", "warp", "lane", "lane_global"][summary["layout"]],
                   "block_size": summary.get("block_size"), "grid_size": summary.get("grid_size"),
                   "lane_update": summary.get("lane_update"),
                   "l2": "flushed between steps (256 MiB write)", "wall_s": wall},
        "e2e": {"value": e2e_value, "unit": "transitions/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_step_ms,
                "path": "mbg_model_parse_strings + mbg_sim_create + mbg_sim_run + mbg_sim_probtraj_sparse + "
                        "TH/final/fixed-point reads", "window_table": ["", "dense", "hash"][summary["window_table"]]},
        "e2e_cold": cold,
        "gpu_launches": 3 * args.steps,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "summary": {k: summary[k] for k in ("transitions", "fixed_points", "finished", "errors", "fixed_point_states")},
    }
    if secondary is not None:
        line["secondary"] = secondary
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="medium", choices=sorted(WORKLOADS) + ["sweep", "surrogate", "l2atomics"])
    ap.add_argument("--layout", type=int, default=0, help="0 autotuned, 1 thread, 2 warp, 3 lane, 4 lane (global rows)")
    ap.add_argument("--block", type=int, default=0, help="threads per block (0: the layout's default); profiling")
    ap.add_argument("--lane-update", type=int, default=0, help="lane layout: 0 cooperative, 1 per lane, 2 per lane with the active words in global memory; profiling")
    ap.add_argument("--window-table", type=int, default=0, help="0 auto, 1 dense, 2 hash table; profiling")
    ap.add_argument("--cpu-seconds", type=float, default=CPU_SAMPLE_SECONDS)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the sweep and surrogate measurements")
    ap.add_argument("--n-traj", type=int, default=0, help="trajectories (default: the workload's); profiling only")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "surrogate":
        import upmabossg_gb300 as mbg
        if mbg.device_count() < 1:
            raise SystemExit("bench: no CUDA device")
        line = measure_surrogate()
        line.update({"n_gpus": 1, "higher_is_better": True, "data": "synthetic", "dtype": "bf16"})
        print(json.dumps(line), flush=True)
        return 0
    if args.workload == "l2atomics":
        # the secondary roofline's denominator: u64 atomic adds per second into L2-resident tables
        import upmabossg_gb300 as mbg
        rates = {str(d): mbg.l2_atomic_rate(d) for d in (1, 32, 1024, 1 << 16, 1 << 20, 1 << 23)}
        print(json.dumps({"metric": "L2 u64 atomic adds/s (no return), by distinct addresses", "unit": "atomics/s",
                          "rates": rates}), flush=True)
        return 0
    if args.workload == "sweep":
        import upmabossg_gb300 as mbg
        if mbg.device_count() < 1:
            raise SystemExit("bench: no CUDA device")
        line = measure_sweep(args.steps, args.warmup)
        line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                     "data": "synthetic", "dtype": "u64"})
        print(json.dumps(line), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
