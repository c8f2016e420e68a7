"""Batched phase-diagram sweep of 2D hexagonal diblock instances (uneven grids 32^2 .. 128^2).

    python polyfields.jl_gb300/sweep_hex.py [--count 256] [--nthreads 32] [--precision fp32]
    torchrun --nproc-per-node N polyfields.jl_gb300/sweep_hex.py ...   # instances sharded by cost

Instance parameters come from one seeded stream (workloads.hex_sweep_params): n ~ U{32, 48,
64, 96, 128}, chiN ~ U[12, 30], fA ~ U[0.25, 0.5], a0 ~ U[4, 9], Ns = 100, seeded noise plus
six-fold cosines.  Each instance runs scft! with AndersonUpdater(nhist = 10) and
DomainUpdater(nskip = 5, nper = 20) (none with --fixed-cell): float32 until ferr < 1e-5,
then float64 polish to ftol = stol = 1e-7 (--precision fp32), or float64 throughout
(--precision fp64).  Instances whose iteration diverges are counted as failed.  Prints
one JSON line with the wall time, instances/s, SCFT iterations/s over all instances and the
convergence count.
"""
import argparse
import json
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from polyfields import sweep as S  # noqa: E402
from polyfields import workloads as W  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--nthreads", type=int, default=32)
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--nsteps", type=int, default=3000)
    ap.add_argument("--fixed-cell", action="store_true", help="no DomainUpdater (cells held at a0)")
    a = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("gloo")
    params = W.hex_sweep_params(a.count, a.seed)
    t0 = time.perf_counter()
    res = S.run_sharded(params, rank, world, precision=a.precision, nsteps=a.nsteps, nthreads=a.nthreads,
                        vcell=not a.fixed_cell)
    wall = time.perf_counter() - t0
    if rank == 0:
        iters = sum(r["iterations"] for r in res)
        by_n = {}
        for p, r in zip(params, res):
            by_n.setdefault(p["n"], []).append(r["iterations"])
        print(json.dumps({
            "workload": f"{a.count} hexagonal diblock instances, grids 32^2..128^2, Ns 100, nhist 10, "
                        + ("fixed cells, ftol=1e-7" if a.fixed_cell else "nskip 5 nper 20, ftol=stol=1e-7"),
            "precision": "fp32 then fp64 polish" if a.precision == "fp32" else "fp64",
            "n_ranks": world, "nthreads": a.nthreads, "wall_s": wall, "instances_per_s": a.count / wall,
            "scft_iters_total": iters, "scft_iters_per_s": iters / wall,
            "converged": sum(1 for r in res if r["converged"]), "failed": sum(1 for r in res if r["status"] != 0),
            "mean_iterations_by_grid": {str(k): sum(v) / len(v) for k, v in sorted(by_n.items())},
            "errors": sorted({r["error"] for r in res if r["status"] != 0})[:4]}))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
