"""Times the reference kernels on one synthetic workload: python -m baseline.refgpu <workload> [n_traj]."""
import json
import sys

from upmabossg_gb300 import synth

from . import run

if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "medium"
    # default: the workload's trajectories, but at most 600 000, below the 671 088 at which the
    # reference's window kernel overflows its record index on the 1000-node model
    n = int(sys.argv[2]) if len(sys.argv) > 2 else 0
    net = getattr(synth, name)()
    if n == 0:
        n = min(net.sample_count, 600_000)
    r = run(net.bnd(), net.cfg(), n)
    print(json.dumps({"workload": name, "trajectories": r.n_traj, "transitions": r.transitions,
                      "sim_ms": r.sim_ms, "transitions_per_s": r.transitions / (r.sim_ms * 1e-3),
                      "compile_ms": r.compile_ms, "count_ms": r.count_ms, "launches": r.iterations}))
