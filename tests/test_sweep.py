"""Phase-diagram sweep host logic: cost-balanced sharding over ranks and the result gather.

The multi-rank path runs as two gloo ranks on the CPU with a stand-in runner (no GPU):
every instance must run exactly once, on the rank the partition assigns, and every rank
must end with all results in instance order.
"""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "polyfields.jl_gb300")

from polyfields import sweep as S  # noqa: E402
from polyfields import workloads as W  # noqa: E402


@pytest.mark.parametrize("world", [1, 2, 3, 4])
def test_shard_by_cost_partitions_every_instance_once(world):
    rng = np.random.default_rng(world)
    costs = rng.choice([32**2, 48**2, 64**2, 96**2, 128**2], size=61).astype(float)
    parts = S.shard_by_cost(costs, world)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    # LPT bound: no rank exceeds the mean load by more than the largest single instance
    assert max(loads) <= sum(costs) / world + max(costs) + 1e-9
    assert parts == S.shard_by_cost(costs, world)  # deterministic on every rank


def test_sweep_params_are_seeded_and_in_range():
    a, b = W.hex_sweep_params(64, seed=7), W.hex_sweep_params(64, seed=7)
    assert a == b
    assert a != W.hex_sweep_params(64, seed=8)
    for p in a:
        assert p["n"] in (32, 48, 64, 96, 128)
        assert 0.12 <= p["chi"] <= 0.30
        assert 25 <= p["NA"] <= 50
        assert 4.0 <= p["a0"] <= 9.0


def test_sweep_instance_builds_on_the_oracle():
    """The instance builder runs against the oracle's API (the reference's names): a
    Multiblock of N_A + N_B = 100 in a hexagonal cell, six-fold start."""
    import pf_oracle as O
    p = dict(n=32, chi=0.2, NA=30, a0=6.0, seed=3)
    o = W.hex_instance(O, **p)
    assert o.species[0].N == 100
    o.density_update()
    assert np.isfinite(o.free_energy())
    assert abs(o.density[1].mean() - 0.30) < 1e-12


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, PKG)
    import torch.distributed as dist
    from polyfields import sweep
    from polyfields import workloads
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    params = workloads.hex_sweep_params(23, seed=5)

    def fake_runner(ps, idx):
        return {i: {"n": ps[i]["n"], "rank": rank} for i in idx}

    res = sweep.run_sharded(params, rank, world, runner=fake_runner)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        for r in res:
            f.write(f"{r['n']} {r['rank']}\n")
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_sweep_gathers_all_results_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    params = W.hex_sweep_params(23, seed=5)
    parts = S.shard_by_cost([S.instance_cost(p) for p in params], world)
    owner = {i: r for r, p in enumerate(parts) for i in p}
    for rank in range(world):
        lines = open(os.path.join(str(tmp_path), f"rank{rank}.txt")).read().split("\n")[:-1]
        assert len(lines) == len(params)
        for i, line in enumerate(lines):
            n, r = map(int, line.split())
            assert n == params[i]["n"] and r == owner[i]
