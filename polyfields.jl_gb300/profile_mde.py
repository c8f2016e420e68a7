"""Run a few MDE contour steps for kernel profiling.

    python polyfields.jl_gb300/profile_mde.py [--n 128] [--steps 8] [--precision fp32]
    python polyfields.jl_gb300/profile_mde.py --blend [--n 128] [--steps 20] [--solves 3]

Default: one chain of `steps` RK2 contour steps through pf_propagate on an n^3 cubic grid
(n x n plane kernels, n-point z pencils) with seeded fields.  --blend: `solves` density
solves of the large-blend system (diblock + homopolymer: three chains, one stream each, as in
the benchmark) with Ns = `steps`.  Both keep the device footprint small
(a few hundred MB at 128^3), so a profiler can replay each launch.
"""
import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import polyfields as pf  # noqa: E402
from polyfields import _lib as L  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--blend", action="store_true")
    ap.add_argument("--solves", type=int, default=3)
    a = ap.parse_args()
    n = a.n
    if a.blend:
        from polyfields import workloads as W
        sysm = W.blend3d_system(pf, n=n, precision=a.precision, Ns=a.steps)
        for _ in range(a.solves):
            sysm.density_update()
        sysm.synchronize()
        print("Q after", a.solves, "solves:", [sp.Q for sp in sysm.species])
        return
    sysm = pf.FieldSystem((n, n, n), pf.UnitCell(3, "cubic", 14.0), precision=a.precision)
    rng = np.random.Generator(np.random.PCG64(12345))
    w = 0.05 * rng.standard_normal((n, n, n))
    q0 = np.ones((n, n, n))
    out = np.empty_like(q0)
    lib = L.load()
    for _ in range(2):
        L.check(lib.pf_propagate(sysm._h, L.dptr(w), 1.0, 1.0, 0.5, L.dptr(q0), L.dptr(out), a.steps), sysm._h)
    print("mean q after", a.steps, "steps:", float(out.mean()))


if __name__ == "__main__":
    main()
