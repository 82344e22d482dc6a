"""Sharding across ranks (bench.py under torchrun): each rank simulates its own range of
trajectory ids; because every trajectory is keyed by (seed, id), the ranks' results summed equal
one run over all ids. Checked with two gloo ranks on the CPU, the oracle standing in for each
rank's GPU."""
import os
import socket

import numpy as np
import pytest

import upmabossg_gb300 as mbg


def test_shard_ranges_partition_the_ids():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            ranges = [mbg.shard_range(n, r, world) for r in range(world)]
            ids = [i for b, c in ranges for i in range(b, b + c)]
            assert ids == list(range(n))
    with pytest.raises(ValueError):
        mbg.shard_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, bnd, cfg, frac_bits, n, out):
    import torch
    import torch.distributed as dist

    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    base, count = mbg.shard_range(n, rank, world)
    r = oracle.run(bnd, cfg, frac_bits=frac_bits, n_traj=count, traj_base=base, threads=2)
    hist = torch.from_numpy(r.dense_hist())
    final = torch.from_numpy(r.final.copy())
    trans = torch.tensor([r.counters["transitions"]], dtype=torch.float64)
    for t in (hist, final, trans):
        dist.all_reduce(t)
    if rank == 0:
        np.savez(out, hist=hist.numpy(), final=final.numpy(), trans=trans.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_run(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    import oracle
    from upmabossg_gb300 import synth
    net = synth.sweep_instance(1)  # 56 nodes, 8 outputs
    bnd, cfg = net.bnd(), net.cfg()
    m = mbg.Model.from_strings(bnd, cfg)
    n = 301
    out = str(tmp_path / "r.npz")
    tmp.spawn(_rank_main, args=(2, _free_port(), bnd, cfg, m.info.frac_bits, n, out), nprocs=2, join=True)
    got = np.load(out)
    ref = oracle.run(bnd, cfg, frac_bits=m.info.frac_bits, n_traj=n)
    assert np.allclose(got["hist"], ref.dense_hist(), rtol=1e-12, atol=1e-9)
    assert np.array_equal(got["final"], ref.final)
    assert int(got["trans"][0]) == ref.counters["transitions"]
