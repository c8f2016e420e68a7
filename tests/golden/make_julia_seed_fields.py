"""Regenerate tests/golden/julia_seed_fields.npz: the fields that the reference's seeded
`fieldinit!(sys; scale, seed = 12345)` (src/fileio.jl:14-23) writes in its two RNG-dependent
tests and in the seeded run of its example notebook.

* test/test_system.jl:3-26: grid 32x1x1, monomers with ids 1, 2, 3 -> keys system_w1..3
* test/test_updaters.jl:3-16: grid 32x1x1, monomers with ids 1, 2 -> keys updaters_w1..2
* examples/examples.ipynb cell 11 (the ABC blend, `fieldinit!(sys; scale = 0.05,
  seed = 12345)`): grid 256x1x1, monomers with ids 1, 2, 3 -> keys nbblend_w1..3

Arrays have shape (Nz, Ny, Nx).  The values come from oracle/julia_rng.py, the restatement of
the Julia runtime's seeded `randn` and `Dict` order (it needs mpmath for its ziggurat
tables).  Each case reseeds, so each set starts from seed 12345.

Usage:  python tests/golden/make_julia_seed_fields.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))

import julia_rng  # noqa: E402

SEED = 12345
CASES = {  # name: (monomer ids, grid (Nx, Ny, Nz), scale)
    "system": ((1, 2, 3), (32, 1, 1), 0.1),
    "updaters": ((1, 2), (32, 1, 1), 0.1),
    "nbblend": ((1, 2, 3), (256, 1, 1), 0.05),
}


def fields():
    out = {}
    for name, (mids, dims, scale) in CASES.items():
        for mid, vals in julia_rng.fieldinit_fields(mids, dims, SEED, scale).items():
            out[f"{name}_w{mid}"] = np.array(vals, dtype=np.float64).reshape(dims[2], dims[1], dims[0])
    return out


def main() -> None:
    dst = os.path.join(HERE, "julia_seed_fields.npz")
    np.savez_compressed(dst, **fields())
    print(f"wrote {dst}")


if __name__ == "__main__":
    main()
