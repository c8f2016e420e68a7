"""Time-to-solution of the large-blend system: plain FP64 solve vs FP32 iterations with FP64 polish.

    python polyfields.jl_gb300/converge.py [--n 128] [--nsteps 4000] [--switch 3e-6] [--modes mixed,fp64]
        [--nhist 20] [--iter-euler 1] [--lam-euler 0.01] [--nskip 5] [--nper 20] [--fixed-cell]
        [--system blend|bcc]

--system bcc runs the 3D BCC workload instead (AB diblock fA 0.3, N100, Ns 100, cubic L0 7,
twelve {110} cosines + 0.1 noise).

Builds the large blend (AB diblock N100 fA0.4 at phi 0.8 + A homopolymer N50 at phi 0.2,
chi 0.2, Ns 200, cubic cell L0 = 14, double-gyroid start plus 0.05 seeded noise) on an n^3
grid and runs scft! with AndersonUpdater(nhist = 20) and DomainUpdater(nskip = 5, nper = 20)
to ftol = stol = 1e-8, once with float64 propagators throughout and once with float32
propagators until ferr < --switch followed by float64 iterations (the mixed path).  Prints
one JSON line: wall time, iterations, final ferr/serr/fhelm and cell of each run, and the
differences of the mixed run from the FP64 run (|dfhelm|, |dL|/L).
"""
import argparse
import json
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import polyfields as pf  # noqa: E402
from polyfields import workloads as W  # noqa: E402


def run(n, precision, nsteps, switch, ftol, stol, nsout, a):
    if a.system == "bcc":
        sysm = W.bcc_system(pf, n=n, precision=precision)
    else:
        sysm = W.blend3d_system(pf, n=n, precision=precision)
    sysm.synchronize()
    opts = pf.SCFTOptions(nsteps=nsteps, ftol=ftol, stol=stol, nsout=nsout,
                          mixed_switch_ferr=switch if precision == "fp32" else 0.0)
    upd = pf.AndersonUpdater(nhist=a.nhist, iter_euler=a.iter_euler, lam_euler=a.lam_euler)
    dom = None if a.fixed_cell else pf.DomainUpdater(nskip=a.nskip, nper=a.nper)
    t0 = time.perf_counter()
    r = pf.scft(sysm, upd, domain=dom, opts=opts)
    sysm.synchronize()
    wall = time.perf_counter() - t0
    return {"precision": "mixed" if precision == "fp32" else "fp64", "wall_s": wall, "iterations": r.nsteps,
            "converged": r.converged, "switch_step": r.switch_step, "ferr": r.ferr, "serr": r.serr,
            "fhelm": r.fhelm, "L": float(sysm.cell.params[0])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--nsteps", type=int, default=4000)
    ap.add_argument("--switch", type=float, default=3e-6)
    ap.add_argument("--ftol", type=float, default=1e-8)
    ap.add_argument("--stol", type=float, default=1e-8)
    ap.add_argument("--modes", default="mixed,fp64")
    ap.add_argument("--nsout", type=int, default=0)
    ap.add_argument("--nhist", type=int, default=20)
    ap.add_argument("--iter-euler", type=int, default=1)
    ap.add_argument("--lam-euler", type=float, default=0.01)
    ap.add_argument("--nskip", type=int, default=5)
    ap.add_argument("--nper", type=int, default=20)
    ap.add_argument("--fixed-cell", action="store_true", help="no DomainUpdater (cell held at L0)")
    ap.add_argument("--system", default="blend", choices=["blend", "bcc"])
    a = ap.parse_args()
    cellmode = "fixed cell" if a.fixed_cell else f"DomainUpdater nskip {a.nskip} nper {a.nper}"
    name = "large blend" if a.system == "blend" else "BCC diblock fA0.3 L0 7, Ns 100"
    out = {"workload": f"{name} {a.n}^3, Anderson nhist {a.nhist} (iter_euler {a.iter_euler}, "
                       f"lam_euler {a.lam_euler}), {cellmode}", "ftol": a.ftol, "stol": a.stol,
           "switch_ferr": a.switch, "runs": []}
    for mode in a.modes.split(","):
        prec = "fp32" if mode == "mixed" else "fp64"
        out["runs"].append(run(a.n, prec, a.nsteps, a.switch, a.ftol, a.stol, a.nsout, a))
        print(json.dumps(out["runs"][-1]), file=sys.stderr, flush=True)
    runs = {r["precision"]: r for r in out["runs"]}
    if "mixed" in runs and "fp64" in runs:
        m, d = runs["mixed"], runs["fp64"]
        out["abs_dfhelm"] = abs(m["fhelm"] - d["fhelm"])
        out["rel_dL"] = abs(m["L"] - d["L"]) / abs(d["L"])
        out["wall_speedup"] = d["wall_s"] / m["wall_s"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
