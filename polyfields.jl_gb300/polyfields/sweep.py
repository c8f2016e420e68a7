"""Phase-diagram sweeps: many independent scft! runs, batched on one GPU and sharded over ranks.

Instances are independent, so a multi-GPU sweep needs no device collective: each rank takes
a cost-balanced share of the instances (longest-processing-time-first over the cost grid
points x contour steps), runs it with ``scft_batch`` on its own GPU, and the ranks exchange
only the small per-instance results on the host (``torch.distributed.all_gather_object``).
"""
import time
from typing import Callable, Dict, List, Optional, Sequence


def instance_cost(p: Dict) -> float:
    """Relative cost of one instance: grid points x contour steps per density solve."""
    n = int(p["n"])
    return float(n * n * int(p.get("Ns", 100)))


def shard_by_cost(costs: Sequence[float], world: int) -> List[List[int]]:
    """Greedy longest-processing-time partition of instance indices over ``world`` ranks.

    Instances are taken in decreasing cost (ties by index) and each goes to the rank with
    the smallest load so far (ties to the lower rank); each rank's list is in index order.
    Deterministic, so every rank computes the same partition without communicating."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    loads = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(p) for p in parts]


def run_local(params: Sequence[Dict], indices: Sequence[int], precision: str = "fp32", ftol: float = 1e-7,
              stol: float = 1e-7, switch: float = 1e-5, nsteps: int = 3000, nthreads: int = 0,
              vcell: bool = True, polish: str = "auto") -> Dict[int, Dict]:
    """Run the instances ``indices`` of ``params`` on this process's GPU with scft_batch:
    float32 iterations until ferr < ``switch`` then float64 polish to ``ftol``/``stol``
    (precision "fp32"), or float64 throughout ("fp64").  Returns {index: result dict}."""
    import polyfields as pf
    from polyfields import _lib as L
    from polyfields import workloads as W
    systems, ups, doms = [], [], []
    for i in indices:
        p = params[i]
        systems.append(W.hex_instance(pf, p["n"], p["chi"], p["NA"], p["a0"], p["seed"], precision=precision))
        ups.append(pf.AndersonUpdater(nhist=10))
        doms.append(pf.DomainUpdater(nskip=5, nper=20) if vcell else None)
    opts = pf.SCFTOptions(nsteps=nsteps, ftol=ftol, stol=stol,
                          mixed_switch_ferr=switch if precision == "fp32" else 0.0, polish=polish)
    t0 = time.perf_counter()
    res, st = pf.scft_batch(systems, ups, doms if vcell else None, opts, nthreads=nthreads, raise_on_error=False)
    wall = time.perf_counter() - t0
    out = {}
    lib = L.load()
    for k, i in enumerate(indices):
        r = res[k]
        err = lib.pf_last_error(systems[k]._h).decode() if st[k] != 0 else ""
        out[i] = {"status": int(st[k]), "error": err, "converged": bool(r.converged), "iterations": int(r.nsteps),
                  "ferr": float(r.ferr), "serr": float(r.serr), "fhelm": float(r.fhelm),
                  "switch_step": int(r.switch_step), "a": float(systems[k].cell.params[0]), "wall_s": wall}
    return out


def run_sharded(params: Sequence[Dict], rank: int = 0, world: int = 1,
                runner: Optional[Callable[[Sequence[Dict], Sequence[int]], Dict[int, Dict]]] = None,
                **kw) -> List[Dict]:
    """Run a sweep over ``world`` ranks (``torch.distributed`` initialised when world > 1):
    this rank runs its cost-balanced share with ``runner`` (default ``run_local``), then the
    per-instance results are gathered on every rank.  Returns the results in instance order."""
    parts = shard_by_cost([instance_cost(p) for p in params], world)
    runner = runner or (lambda ps, idx: run_local(ps, idx, **kw))
    mine = runner(params, parts[rank]) if parts[rank] else {}
    if world > 1:
        import torch.distributed as dist
        allr: List[Optional[Dict[int, Dict]]] = [None] * world
        dist.all_gather_object(allr, mine)
    else:
        allr = [mine]
    merged: Dict[int, Dict] = {}
    for d in allr:
        for i, r in (d or {}).items():
            if i in merged:
                raise RuntimeError(f"instance {i} ran on two ranks")
            merged[i] = r
    missing = [i for i in range(len(params)) if i not in merged]
    if missing:
        raise RuntimeError(f"instances {missing[:8]} have no result")
    return [merged[i] for i in range(len(params))]
