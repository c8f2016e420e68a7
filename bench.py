#!/usr/bin/env python
"""Benchmark: SCFT iterations/s of the large blend at 128^3 on one GB300.

Workload (one "step" = one scft! iteration = AndersonUpdater.step!): AB diblock N100 fA0.4
(phi 0.8) + A homopolymer N50 (phi 0.2), chi 0.2, Ns 200, 128^3 grid, cubic cell L0 14,
double-gyroid start + 0.05 seeded noise, Anderson nhist 20.  One iteration is one density
solve -- 600 MDE contour steps (diblock forward + backward, homopolymer forward), Simpson
integration, residuals -- and the Anderson Gram/solve/mix.  The timed region runs the FP32
propagators of the mixed-precision path (densities, residuals, Gram and solve in FP64); the
FP64 propagator rate is measured after it on the same state.

  python bench.py [--steps K] [--warmup W]            # GPU engine (one JSON line)
  python bench.py --impl reference [--steps K ...]    # the FP64 CPU restatement (oracle)
  python bench.py --mode tts [--size N] [--seeds S]   # time to solution: mixed vs plain FP64
  python bench.py --mode sweep [--count 256]          # batched 2D hexagonal phase-diagram sweep
  python bench.py --mode profile [--size N] [--ns NS] # a few density solves, small, for ncu

Inputs are synthetic (seeded NumPy PCG64 fields of the benchmark's shapes) and the working
set (propagator histories, ~5 GB) is far larger than the 129 MB L2.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "polyfields.jl_gb300"))

N_GRID = 128
MDE_STEPS_PER_ITER = 600  # 200 (diblock q) + 200 (diblock qc) + 200 (homopolymer q)
METRIC = "SCFT iters/s at 128^3 (mixed path: FP32 propagators, FP64 reductions/Anderson)"
UNIT = "iters/s"
NHIST = 20
WORKLOAD = {
    "workload": "large blend 128^3: AB diblock N100 fA0.4 phi0.8 + A homopolymer N50 phi0.2, chi0.2, Ns200, "
                "cubic L0=14, double-gyroid init, Anderson nhist20",
    "grid": [N_GRID, N_GRID, N_GRID],
    "mde_steps_per_iter": MDE_STEPS_PER_ITER,
    "l2_policy": "inputs larger than L2 (propagator histories ~5 GB per iteration)",
    "anderson_history": "full (20 entries) before the warm-up and timed steps",
}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms during the timed region (the
    timed region starts after the first sample has arrived)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for name, flag in zip(names, parts[5:9]):
                    if flag.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_blend(n=N_GRID, seed=12345):
    """The benchmark workload held by the C++/OpenMP FP64 CPU restatement (oracle/pf_cpu.cpp), on
    all host threads, with the Anderson updater (nhist 20) set up."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pf_cpu as C
    import pf_oracle as O
    from polyfields import workloads as W
    o = W.blend3d_system(O, n=n, inject=False)  # configuration only: no NumPy density solve
    c = C.CpuSystem.from_oracle(o)
    for mid, w in W.blend3d_fields(n, seed).items():
        c.set_field(mid, w)
    del o
    c.anderson_setup(NHIST)
    return c


CPU_KIND = "port"
CPU_SAMPLE = ("one scft! iteration of the 128^3 blend (density: 600 contour steps with the project's FFT, Simpson, "
              "residuals, free energy, field error; Anderson step) in the C++17/OpenMP FP64 CPU restatement "
              "(oracle/pf_cpu.cpp)")


def cpu_baseline_sample(warm=1, timed=1):
    """The C++/OpenMP FP64 CPU restatement on a bounded sample of the same workload: `timed` full
    SCFT iterations (after `warm` untimed ones: the first is the Anderson updater's Euler step)
    on all host threads.  The Anderson history then holds `warm` entries, so the Gram sums of a
    full 20-entry history (under 2% of an iteration here) are not in the sample."""
    c = cpu_blend()
    for _ in range(warm):
        c.anderson_step()
    t0 = time.perf_counter()
    for _ in range(timed):
        c.anderson_step()
        c.free_energy()
        c.field_error()
    dt = (time.perf_counter() - t0) / timed
    return {"value": 1.0 / dt, "unit": UNIT, "cores": c.threads, "kind": CPU_KIND,
            "sample": f"{timed} x " + CPU_SAMPLE + f" after {warm} warm-up iteration(s): {dt:.1f} s per iteration",
            "mde_steps_per_s": MDE_STEPS_PER_ITER / dt}


def run_reference(args):
    """Reference arm: the reference (Julia + FFTW) cannot run here, so this times its FP64 CPU
    restatement in C++/OpenMP (oracle/pf_cpu.cpp) on all host threads, one full scft!
    iteration of the benchmark workload per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    c = cpu_blend()
    for _ in range(max(1, args.warmup)):
        c.anderson_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.anderson_step()
        c.free_energy()
        c.field_error()
    dt = time.perf_counter() - t0
    value = args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(WORKLOAD, size=N_GRID),
            "mde_steps_per_s": value * MDE_STEPS_PER_ITER,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": c.threads, "kind": CPU_KIND,
                             "sample": CPU_SAMPLE + " per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def replica_env():
    """(rank, world) of this process under torchrun (1 GPU per rank), else (0, 1)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def pin_replica_gpu():
    """Under torchrun with several ranks, make this rank see only its own GPU (LOCAL_RANK-th of
    the visible ones) before CUDA starts: every rank then runs one independent instance on its
    device 0 (a single SCFT instance does not shard: each contour step is a full 3D FFT)."""
    rank, world = replica_env()
    if world <= 1:
        return
    local = int(os.environ.get("LOCAL_RANK", rank))
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    devs = [d for d in vis.split(",") if d.strip()] if vis else None
    os.environ["CUDA_VISIBLE_DEVICES"] = devs[local % len(devs)] if devs else str(local)


def replica_group():
    """Host process group (gloo) of the replicas, or None when running alone."""
    rank, world = replica_env()
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    return dist


def aggregate_replicas(dist, ms_total, units):
    """Whole-job rate of `units` per rank over the slowest rank's time: (world * units) /
    max(ms_total) per second, and that max (ms).  dist None: one rank."""
    if dist is None:
        return 1000.0 * units / ms_total, ms_total
    import torch
    t = torch.tensor([float(ms_total)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    mx = float(t.item())
    return 1000.0 * units * dist.get_world_size() / mx, mx


def run_gpu(args):
    import numpy as np
    import polyfields as pf
    from polyfields import _lib as L
    from polyfields.workloads import blend3d_system

    lib = L.load()
    rank, world = replica_env()
    if args.gpus != world:
        raise SystemExit(f"--gpus {args.gpus} but {world} rank(s): launch N ranks with torchrun for --gpus N")
    dist = replica_group()  # N > 1: N independent replicas (no data-path collective)
    n = args.size
    sysm = blend3d_system(pf, n=n, precision="fp32")
    ng = n ** 3
    # the initial state's free energy: tests/test_gpu_parity_large.py checks this state (both
    # precisions) against the FP64 oracle
    fhelm_initial = sysm.free_energy()
    upd = pf.AndersonUpdater(nhist=NHIST)
    upd.setup(sysm)
    sysm.set_timing(True)
    # Fill the Anderson history (nhist entries) before the warm-up steps, so that the timed
    # iterations are steady-state ones: the Gram step's cost grows with the history length.
    for _ in range(NHIST):
        upd.step()
    for _ in range(args.warmup):
        upd.step()
    sysm.synchronize()

    # ---- timed region: K scft! iterations with FP32 propagators
    clocks = ClockSampler()
    if rank == 0:
        clocks.start()
    if dist is not None:
        dist.barrier()
    l0 = lib.pf_launch_count()
    prop_ms = 0.0
    dens_ms = 0.0
    L.check(lib.pf_record_event(sysm._h, 0), sysm._h)
    t_host = time.perf_counter()
    for _ in range(args.steps):
        upd.step()
        a, b, nmde = sysm.last_timing()
        prop_ms += a
        dens_ms += b
    L.check(lib.pf_record_event(sysm._h, 1), sysm._h)
    import ctypes
    ms = ctypes.c_double()
    L.check(lib.pf_elapsed_ms(sysm._h, 0, 1, ctypes.byref(ms)), sysm._h)
    t_host = time.perf_counter() - t_host
    launches = lib.pf_launch_count() - l0
    clk = clocks.stop() if rank == 0 else None
    value, ms_max = aggregate_replicas(dist, ms.value, args.steps)
    ms_per_step = ms_max / args.steps
    prop_step_ms = prop_ms / args.steps
    mde_step_us = 1000.0 * prop_step_ms / nmde
    ferr = sysm.field_error()
    fhelm = sysm.free_energy()
    sysm_schedule = sysm.pencil_schedule()

    # ---- roofline of the dominant kernel pair (one MDE contour step: xy_step + z_pipe)
    peak, peak_kind = measured_peaks()
    alg_bytes = 3 * 4 * ng  # read q_s (f32), read LW (f32), write q_{s+1} (f32)
    achieved = alg_bytes / (mde_step_us * 1e-6) / 1e9
    # DRAM bytes of one contour step of one chain at 128^3 (xy_step + z_pipe launches) from an
    # ncu capture of the large blend with Ns = 20 (bench.py --mode profile): reads 16.96 MB +
    # 12.81 MB, writes 0 (absorbed by L2 within the launch); cold caches.
    traffic = 29.77e6 if n == 128 else None
    roofline = {"bound": "hbm", "kernel": "MDE contour step (xy_step_kernel<float,128,128> + z_pipe_kernel<float,128>)",
                "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                "avg_step_us": mde_step_us}
    # The step is issue bound before it is HBM bound: ncu counts 4.91e6 + 1.66e6 warp instructions
    # for one chain step at 128^3 (plane + pencil pass, same capture); 152 SMs x 4 schedulers issue
    # at most one warp instruction per cycle each at the sampled SM clock.
    issue = None
    if n == 128:
        winst = 4.91e6 + 1.66e6
        mhz = (clk or {}).get("sm_mhz") or 2070.0
        floor_us = winst / (152 * 4 * mhz * 1e6) * 1e6
        issue = {"warp_instructions_per_step": winst, "floor_us": floor_us, "frac": floor_us / mde_step_us}

    # ---- e2e through the public API with host buffers (pinned when torch is present)
    try:
        import torch
        host = {m: torch.empty((n, n, n), dtype=torch.float64, pin_memory=True).numpy() for m in (1, 2)}
    except Exception:
        host = {m: np.empty((n, n, n)) for m in (1, 2)}
    for m in (1, 2):
        host[m][...] = sysm.fields[m]
    e2e_steps = max(1, min(args.steps, 5))
    sysm.synchronize()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for m in (1, 2):
            L.check(lib.pf_set_field(sysm._h, m, L.dptr(host[m])), sysm._h)
        upd.step()
        for m in (1, 2):
            L.check(lib.pf_get_grid(sysm._h, L.PF_FIELD, m, L.dptr(host[m])), sysm._h)
        _ = sysm.free_energy()
    e2e_value, _ = aggregate_replicas(dist, 1000.0 * (time.perf_counter() - t0), e2e_steps)
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": world * 2 * 8 * ng,
           "d2h_bytes_per_step": world * (2 * 8 * ng + 8),
           "api": "pf_set_field x2 + pf_anderson_step + pf_get_grid x2 + pf_free_energy"}
    if rank != 0:
        return 0

    # ---- FP64 propagators on the same state (the plain FP64 GPU solver's iteration rate; one
    # GPU, so only when the benchmark runs alone)
    fp64 = None
    if args.fp64_steps > 0 and world == 1:
        sysm.precision = "fp64"
        upd.step()
        L.check(lib.pf_record_event(sysm._h, 2), sysm._h)
        for _ in range(args.fp64_steps):
            upd.step()
        L.check(lib.pf_record_event(sysm._h, 3), sysm._h)
        m64 = ctypes.c_double()
        L.check(lib.pf_elapsed_ms(sysm._h, 2, 3, ctypes.byref(m64)), sysm._h)
        a64, _, _ = sysm.last_timing()
        fp64 = {"iters_per_s": 1000.0 * args.fp64_steps / m64.value, "ms_per_iter": m64.value / args.fp64_steps,
                "mde_step_us": 1000.0 * a64 / nmde, "steps": args.fp64_steps}
        # the same iteration end to end through the C ABI with host fields (as `e2e` above), the
        # like-for-like figure against the FP64 CPU restatement
        for m in (1, 2):
            L.check(lib.pf_get_grid(sysm._h, L.PF_FIELD, m, L.dptr(host[m])), sysm._h)
        sysm.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            for m in (1, 2):
                L.check(lib.pf_set_field(sysm._h, m, L.dptr(host[m])), sysm._h)
            upd.step()
            for m in (1, 2):
                L.check(lib.pf_get_grid(sysm._h, L.PF_FIELD, m, L.dptr(host[m])), sysm._h)
            _ = sysm.free_energy()
        fp64["e2e_iters_per_s"] = e2e_steps / (time.perf_counter() - t0)

    # the CPU baseline and the time to solution run with the benchmark alone (N = 1)
    cpu = cpu_baseline_sample() if args.cpu_seconds > 0 and world == 1 else None
    del upd, sysm
    # time to solution, mixed vs plain FP64, on a grid that fits the run's time (median of seeds)
    tts = (tts_summary(args.tts_size, [12345 + 1000 * i for i in range(args.seeds)])
           if args.tts_size > 0 and world == 1 else None)
    config = dict(WORKLOAD, size=n, parallelism=("replicas: one independent instance per GPU" if world > 1 else "1 GPU"))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 propagators + f64 reductions", "data": "synthetic", "config": config,
            "mde_steps_per_s": value * nmde, "mde_steps_per_iter": nmde, "propagate_ms_per_iter": prop_step_ms,
            "density_ms_per_iter": dens_ms / args.steps, "host_ms_per_step": 1000.0 * t_host / args.steps,
            "fp64": fp64, "mixed_vs_fp64_iter_speedup": (value / fp64["iters_per_s"]) if fp64 else None,
            "ferr": ferr, "fhelm": fhelm, "fhelm_initial": fhelm_initial, "roofline": roofline, "issue_roofline": issue, "e2e": e2e,
            "gpu_launches": int(launches), "pencil_schedule": dict(zip(("stages", "rounds", "autotuned"),
                                                                       sysm_schedule)),
            "clocks": clk, "cpu_baseline": cpu, "time_to_solution": tts}
    print(json.dumps(line))
    return 0


def tts_pair(n, seed, ftol=1e-8, nsteps=4000, switch=3e-3, nhist=NHIST):
    """Time to solution of the large blend on an n^3 grid (cell held at L0 = 14, seeded start):
    scft! with float64 propagators throughout, and the mixed path (float32 propagators until
    ferr < switch, then float64 polish), both to ftol.  Wall time of each pf_scft call."""
    import polyfields as pf
    from polyfields import workloads as W
    out = {}
    for mode in ("fp64", "mixed"):
        sysm = W.blend3d_system(pf, n=n, precision="fp64" if mode == "fp64" else "fp32", seed=seed)
        sysm.synchronize()
        opts = pf.SCFTOptions(nsteps=nsteps, ftol=ftol, mixed_switch_ferr=switch if mode == "mixed" else 0.0)
        t0 = time.perf_counter()
        r = pf.scft(sysm, pf.AndersonUpdater(nhist=nhist), opts=opts)
        sysm.synchronize()
        out[mode] = {"wall_s": time.perf_counter() - t0, "iterations": r.nsteps, "converged": bool(r.converged),
                     "switch_step": r.switch_step, "ferr": r.ferr, "fhelm": r.fhelm,
                     "polish_fp64_solves": r.polish_fp64_solves, "polish_fp32_solves": r.polish_fp32_solves}
        del sysm
    out["wall_ratio"] = out["fp64"]["wall_s"] / out["mixed"]["wall_s"]
    out["abs_dfhelm"] = abs(out["mixed"]["fhelm"] - out["fp64"]["fhelm"])
    return out


def tts_summary(n, seeds):
    runs = [dict(seed=sd, **tts_pair(n, sd)) for sd in seeds]
    ratios = sorted(r["wall_ratio"] for r in runs)
    return {"workload": f"large blend {n}^3 (cell held at L0 = 14), Anderson nhist {NHIST}, ftol 1e-8; mixed = "
                        f"float32 propagators to ferr 3e-3, then Newton-Krylov polish (float64 residuals, "
                        f"float32 Jacobian products)",
            "seeds": list(seeds), "wall_ratio_median": statistics.median(ratios),
            "wall_ratio_min": ratios[0], "wall_ratio_max": ratios[-1],
            "abs_dfhelm_max": max(r["abs_dfhelm"] for r in runs),
            "all_converged": all(r["fp64"]["converged"] and r["mixed"]["converged"] for r in runs), "runs": runs}


def run_tts(args):
    """Time to solution, mixed vs plain FP64, over several seeds (median and spread)."""
    seeds = [12345 + 1000 * i for i in range(args.seeds)]
    line = {"mode": "tts", "metric": "wall-time ratio FP64 / mixed to ftol 1e-8 (|dfhelm| <= 1e-8)",
            "unit": "x", "higher_is_better": True}
    line.update(tts_summary(args.size, seeds))
    line["value"] = line["wall_ratio_median"]
    print(json.dumps(line))
    return 0


def run_profile(args):
    """A small device footprint for profilers: `solves` density solves of the large blend on an
    n^3 grid with Ns = args.ns contour steps per chain (three chains, one stream each, as in the
    benchmark), so that ncu can replay every launch."""
    import polyfields as pf
    from polyfields import workloads as W
    sysm = W.blend3d_system(pf, n=args.size, precision=args.precision, Ns=args.ns)
    for _ in range(args.solves):
        sysm.density_update()
    sysm.synchronize()
    print(json.dumps({"mode": "profile", "grid": args.size, "Ns": args.ns, "solves": args.solves,
                      "precision": args.precision, "Q": [sp.Q for sp in sysm.species]}))
    return 0


def run_sweep(args):
    """Batched phase-diagram sweep of 2D hexagonal diblock instances (grids 32^2 .. 128^2, chiN ~
    U[12, 30], fA ~ U[0.25, 0.5], a0 ~ U[4, 9], Ns 100, seeded noise plus six-fold cosines; one
    seeded parameter stream): scft! with AndersonUpdater(nhist = 10), cells held fixed
    (--sweep-domain: DomainUpdater(nskip = 5, nper = 20)), float32 until ferr < --switch
    (1e-5) then float64 polish (--polish) to ftol = 1e-7 (--precision fp32) or float64
    throughout.  Under torchrun the instances are sharded over the ranks by cost and gathered
    on rank 0."""
    from polyfields import sweep as S
    from polyfields import workloads as W
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:  # each rank sees only its own GPU (pin_replica_gpu)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    params = W.hex_sweep_params(args.count, 12345)
    t0 = time.perf_counter()
    res = S.run_sharded(params, rank, world, precision=args.precision, nsteps=3000, nthreads=args.nthreads,
                        vcell=args.sweep_domain, polish=args.polish, switch=args.switch)
    wall = time.perf_counter() - t0
    if rank == 0:
        iters = sum(r["iterations"] for r in res)
        print(json.dumps({
            "mode": "sweep", "metric": "instances/s", "value": args.count / wall, "unit": "instances/s",
            "workload": f"{args.count} hexagonal diblock instances, grids 32^2..128^2, Ns 100, nhist 10, "
                        + ("nskip 5 nper 20, ftol=stol=1e-7" if args.sweep_domain else "fixed cells, ftol=1e-7"),
            "precision": "fp32 then fp64 polish" if args.precision == "fp32" else "fp64", "polish": args.polish,
            "switch_ferr": args.switch,
            "n_ranks": world, "nthreads": args.nthreads, "wall_s": wall, "scft_iters_total": iters,
            "scft_iters_per_s": iters / wall, "converged": sum(1 for r in res if r["converged"]),
            "failed": sum(1 for r in res if r["status"] != 0),
            "errors": sorted({r["error"] for r in res if r["status"] != 0})[:4]}))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 40 SCFT iterations on the GPU, about 0.4 s, so that the "
                         "100 ms clock sampler sees several samples; 10 for --impl reference)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=N_GRID, help="grid points per axis (default 128)")
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=1.0, help="CPU baseline sample (0: skip; else one iteration)")
    ap.add_argument("--mode", default="iter", choices=["iter", "tts", "sweep", "profile"])
    ap.add_argument("--seeds", type=int, default=3, help="tts: seeds of the time-to-solution runs")
    ap.add_argument("--tts-size", type=int, default=64,
                    help="iter: grid of the time-to-solution leg (0: skip); tts mode uses --size")
    ap.add_argument("--precision", default="fp32", help="profile / sweep: fp32 (mixed) or fp64")
    ap.add_argument("--ns", type=int, default=20, help="profile: contour steps per chain")
    ap.add_argument("--solves", type=int, default=3, help="profile: density solves")
    ap.add_argument("--count", type=int, default=256, help="sweep: instances")
    ap.add_argument("--nthreads", type=int, default=64, help="sweep: host threads")
    ap.add_argument("--sweep-domain", action="store_true", help="sweep: variable cells (DomainUpdater)")
    ap.add_argument("--polish", default="auto", choices=["auto", "updater", "newton"],
                    help="sweep: float64 phase of the mixed runs (SCFTOptions.polish)")
    ap.add_argument("--switch", type=float, default=1e-5, help="sweep: ferr at which the mixed runs switch to float64")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 10 if args.impl == "reference" else 40
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "profile":
        return run_profile(args)
    if args.mode == "sweep":
        return run_sweep(args)
    if args.mode == "tts":
        return run_tts(args)
    return run_gpu(args)


if __name__ == "__main__":
    if "--impl" not in sys.argv:
        pin_replica_gpu()
    sys.exit(main())
