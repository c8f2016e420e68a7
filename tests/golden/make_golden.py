"""Regenerate the golden fixtures under tests/golden/ from the reference checkout.

The reference (PolyFields.jl) ships three converged field seeds under examples/seeds/
(JSON, nested [z][y][x] lists, written by ``savefields``, src/fileio.jl:77-97).  Its
example notebook loads each seed and prints the resulting ``SCFTResults``
(examples/examples.ipynb, cells 4, 8 and 12); the README prints the converged lamellar
run of its usage section (README.md:62-79).  This script converts the seeds to compact
``.npz`` arrays, shape (Nz, Ny, Nx), so that the tests can run where the reference
checkout is absent.  The published scalars the tests compare against are constants in
``tests/golden/reference_values.py`` with the file and cell they come from.

Usage:  python tests/golden/make_golden.py path/to/PolyFields.jl
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def convert(src: str, dst: str) -> None:
    with open(src) as fh:
        raw = json.load(fh)
    grid = [int(g) for g in raw["grid"]]
    arrays = {}
    for mid in raw["mids"]:
        arr = np.array(raw["fields"][str(mid)], dtype=np.float64)
        arrays[f"w{int(mid)}"] = arr.reshape(grid[2], grid[1], grid[0])
    np.savez_compressed(dst, grid=np.array(grid), cell_params=np.array(raw["cell_params"], dtype=np.float64),
                        dim=np.array(int(raw["dim"])), crystal=np.array(raw["crystal"]), **arrays)
    print(f"wrote {dst}: grid {grid}, crystal {raw['crystal']}, params {raw['cell_params']}")


def main() -> None:
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py path/to/PolyFields.jl")
    ref = sys.argv[1]
    for name in ("lam1d", "cyl2d", "abc_blend_1d"):
        convert(os.path.join(ref, "examples", "seeds", f"{name}.json"), os.path.join(HERE, f"seed_{name}.npz"))


if __name__ == "__main__":
    main()
