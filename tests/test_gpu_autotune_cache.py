"""The autotuned launch shape persists on disk: a second process with the same model size class
finds it (no pilot runs) and runs the same shape."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = """
import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth
net = synth.sweep_instance(2)
m = mbg.Model.from_strings(net.bnd(), net.cfg())
s = mbg.Simulation(m, n_traj=20000).run().summary()
print(s["layout"], s["block_size"], s["lane_update"], s["transitions"])
"""


def child(cache_dir):
    env = dict(os.environ, MBG_JIT_CACHE=str(cache_dir), MBG_AUTOTUNE_LOG="1")
    env.pop("MBG_AUTOTUNE_NOCACHE", None)
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    pilots = [ln for ln in r.stderr.splitlines() if ln.startswith("mbg autotune:")]
    return r.stdout.strip().splitlines()[-1], pilots


def test_second_process_uses_the_stored_shape(tmp_path):
    first, pilots1 = child(tmp_path)
    assert pilots1, "the first process times the pilots"
    lines = (tmp_path / "autotune_v2.txt").read_text().splitlines()
    assert len(lines) == 1 and len(lines[0].split()) == 4  # key, layout, block, reader update
    second, pilots2 = child(tmp_path)
    assert pilots2 == [], "the second process found the stored shape"
    assert second == first
