"""bench.py --gpus N: N independent replicas of the single-GPU benchmark, one per rank (a single
SCFT instance does not shard).  Host logic only, on the CPU: each rank is pinned to its own GPU
before CUDA starts, and the whole-job rate is the units of all ranks over the slowest rank's
time, agreed on every rank (two gloo ranks)."""
import importlib.util
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_each_rank_sees_its_own_gpu(monkeypatch):
    B = _bench()
    monkeypatch.setenv("WORLD_SIZE", "4")
    monkeypatch.setenv("RANK", "2")
    monkeypatch.setenv("LOCAL_RANK", "2")
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    B.pin_replica_gpu()
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "6"
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    B.pin_replica_gpu()
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "2"


def test_one_rank_leaves_the_devices_alone(monkeypatch):
    B = _bench()
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "0,1")
    B.pin_replica_gpu()
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "0,1"
    assert B.aggregate_replicas(None, 500.0, 10) == (20.0, 500.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world)})
    B = _bench()
    dist = B.replica_group()
    # rank r took 100 (r + 1) ms for its 10 iterations: the job is bound by the slowest rank
    value, mx = B.aggregate_replicas(dist, 100.0 * (rank + 1), 10)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{value} {mx}\n")
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_rate_is_all_units_over_the_slowest_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for rank in range(world):
        value, mx = map(float, open(os.path.join(str(tmp_path), f"rank{rank}.txt")).read().split())
        assert mx == pytest.approx(200.0)
        assert value == pytest.approx(1000.0 * 10 * world / 200.0)
