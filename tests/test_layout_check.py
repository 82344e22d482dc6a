"""Host-side check of the device tables (mbg_model_layout_check): every index the kernels read —
node, regulator and dependency ids, table, palette and side-record offsets — lies inside the array
it indexes. It runs without a GPU, on every model family the GPU tests simulate, so that an index
the kernels would read out of bounds shows up here as an error rather than on the device."""
import numpy as np
import pytest

import upmabossg_gb300 as mbg
from upmabossg_gb300 import synth

from helpers import golden_model, mixed_network
from test_gpu_parity import wide_network


def models():
    for name in ("cellcycle", "metastasis", "sizek", "montagud"):
        yield name, golden_model(name)
    yield "mixed", mixed_network()
    yield "mixed_discrete", mixed_network(n=80, seed=9, discrete=True)
    yield "wide", wide_network()
    for nm in ("small", "medium", "large"):
        net = getattr(synth, nm)()
        yield nm, (net.bnd(), net.cfg())
    for i in (0, 2, 13):
        net = synth.sweep_instance(i)
        yield f"sweep{i}", (net.bnd(), net.cfg())


@pytest.mark.parametrize("name,src", list(models()), ids=lambda v: v if isinstance(v, str) else "")
def test_layout_indices_in_range(name, src):
    bnd, cfg = src
    m = mbg.Model.from_strings(bnd, cfg)
    m.layout_check()


def test_derived_models_layouts_in_range():
    net = synth.medium()
    m = mbg.Model.from_strings(net.bnd(), net.cfg())
    rng = np.random.default_rng(1)
    m.with_rate_scales(rng.uniform(0.1, 10, m.info.nodes), rng.uniform(0.1, 10, m.info.nodes)).layout_check()
    m.with_mutations({m.names[3]: "ON", m.names[400]: "OFF"}).layout_check()
    bnd, cfg = mixed_network()
    mx = mbg.Model.from_strings(bnd, cfg)
    mx.with_mutations({mx.names[i]: ("ON" if i % 2 else "OFF") for i in range(0, 40, 5)}).layout_check()
