"""Workload builders: the benchmark and test systems, with seeded synthetic fields.

Each builder takes an API module as its first argument -- this package, or any module that
exposes the reference's names (Monomer, Diblock, UnitCell, FieldSystem, FloryInteraction,
fieldinit) -- and returns a system whose fields were injected with fieldinit(sys, Dict)
semantics (src/fileio.jl:25-54).  Inputs are NumPy PCG64 streams, so every caller builds
bit-identical fields.
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "tests", "golden")


def _fs(M, dims, cell, mons, precision):
    if precision is None:
        return M.FieldSystem(dims, cell, monomers=mons)
    return M.FieldSystem(dims, cell, monomers=mons, precision=precision)


def seeded_fields(shape, mids, seed=12345, scale=0.1, pattern=None):
    """Seeded Gaussian noise (NumPy PCG64) plus an optional ordered pattern for mids[0] and
    its negative for mids[1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = {m: scale * rng.standard_normal(shape) for m in mids}
    if pattern is not None:
        out[mids[0]] = out[mids[0]] + pattern
        out[mids[1]] = out[mids[1]] - pattern
    return out


def diblock_system(M, dims, crystal, params, N=100, f=0.5, chi=0.2, Ns=100, precision=None, seed=12345,
                   scale=0.1, amp=0.5):
    A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
    cell = M.UnitCell(sum(1 for d in dims if d > 1), crystal, *params)
    sys = _fs(M, dims, cell, [A, B], precision)
    sys.add_species(M.Diblock(A, B, N, f, 1.0, 1.0, Ns), 1.0)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, chi)
    sys.add_interaction(itx)
    shape = (dims[2], dims[1], dims[0])
    z, y, x = np.meshgrid(*(np.arange(n) / n for n in shape), indexing="ij")
    pattern = amp * (np.cos(2 * np.pi * x) + (np.cos(2 * np.pi * y) if dims[1] > 1 else 0)
                     + (np.cos(2 * np.pi * z) if dims[2] > 1 else 0))
    M.fieldinit(sys, seeded_fields(shape, [1, 2], seed, scale, pattern))
    return sys


def blend_seed_system(M, precision=None):
    """examples/seeds/abc_blend_1d.json with the notebook's blend (examples.ipynb cell 11)."""
    d = np.load(os.path.join(GOLDEN, "seed_abc_blend_1d.npz"))
    A, B, C = M.Monomer(1, 2.0), M.Monomer(2, 2.0), M.Monomer(3, 1.0)
    cell = M.UnitCell(int(d["dim"]), str(d["crystal"]), *d["cell_params"])
    sys = _fs(M, tuple(int(g) for g in d["grid"]), cell, [A, B, C], precision)
    sys.add_species(M.Point(C), 0.4)
    sys.add_species(M.Homopolymer(A, 100, 1.0), 0.3)
    sys.add_species(M.Homopolymer(B, 100, 1.0), 0.3)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.5)
    itx.set_interaction(A, C, 1.25)
    itx.set_interaction(B, C, 1.25)
    sys.add_interaction(itx)
    M.fieldinit(sys, {int(k[1:]): d[k] for k in d.files if k.startswith("w")})
    return sys


def cyl2d_seed_system(M, precision=None):
    """examples/seeds/cyl2d.json with the notebook's cylinder system (examples.ipynb cell 7)."""
    d = np.load(os.path.join(GOLDEN, "seed_cyl2d.npz"))
    A, B = M.Monomer(1), M.Monomer(2)
    cell = M.UnitCell(2, "hexagonal", *d["cell_params"])
    sys = _fs(M, tuple(int(g) for g in d["grid"]), cell, [A, B], precision)
    sys.add_species(M.Diblock(A, B, 100, 0.3, 1.0, 1.0, 100), 1.0)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.3)
    sys.add_interaction(itx)
    M.fieldinit(sys, {int(k[1:]): d[k] for k in d.files if k.startswith("w")})
    return sys


def blend3d_fields(n=32, seed=12345):
    """Start fields of the large-blend workload: the double gyroid sin x cos y + sin y cos z +
    sin z cos x (x = 2 pi X / L) for w_A, its negative for w_B, plus 0.05 seeded noise."""
    shape = (n, n, n)
    z, y, x = np.meshgrid(*(2 * np.pi * np.arange(n) / n for _ in range(3)), indexing="ij")
    gyr = np.sin(x) * np.cos(y) + np.sin(y) * np.cos(z) + np.sin(z) * np.cos(x)
    return seeded_fields(shape, [1, 2], seed, 0.05, gyr)


def blend3d_system(M, n=32, L=14.0, precision=None, Ns=200, seed=12345, inject=True):
    """The large-blend workload (128^3 at full size): AB diblock N100 fA0.4 (phi 0.8) + A
    homopolymer N50 (phi 0.2), chi 0.2, Ns 200, cubic cell L0 = 14, double-gyroid start
    (blend3d_fields).  inject=False returns the system before fieldinit (no density solve)."""
    A, B = M.Monomer(1), M.Monomer(2)
    cell = M.UnitCell(3, "cubic", L)
    sys = _fs(M, (n, n, n), cell, [A, B], precision)
    sys.add_species(M.Diblock(A, B, 100, 0.4, 1.0, 1.0, Ns), 0.8)
    sys.add_species(M.Homopolymer(A, 50, 1.0, Ns), 0.2)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys.add_interaction(itx)
    if inject:
        M.fieldinit(sys, blend3d_fields(n, seed))
    return sys


def hex_sweep_params(count=256, seed=12345):
    """Parameters of a 2D hexagonal phase-diagram sweep, all drawn from one PCG64 stream:
    grid n ~ U{32, 48, 64, 96, 128}, chiN ~ U[12, 30] (N = 100), fA ~ U[0.25, 0.50] with
    N_A = round(100 fA) (chains built as Multiblock([A, B], [N_A, 100 - N_A]): Diblock's float
    truncation misplaces some fA), cell a0 ~ U[4, 9], and a per-instance field seed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.array([32, 48, 64, 96, 128])
    out = []
    for i in range(count):
        n = int(sizes[rng.integers(0, len(sizes))])
        chin = float(rng.uniform(12.0, 30.0))
        fa = float(rng.uniform(0.25, 0.50))
        a0 = float(rng.uniform(4.0, 9.0))
        out.append(dict(n=n, chi=chin / 100.0, NA=int(round(100 * fa)), a0=a0, seed=int(rng.integers(0, 2**31 - 1))))
    return out


def hex_instance(M, n, chi, NA, a0, seed, precision=None, Ns=100, scale=0.1, amp=1.0):
    """One sweep instance: AB diblock (N = 100) in a 2D hexagonal cell on an n x n grid, with
    seeded noise plus the six first-order cosines (reciprocal vectors (1,0), (0,1), (1,1) of
    the 60-degree basis) for w_A and their negative for w_B."""
    A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
    sys = _fs(M, (n, n, 1), M.UnitCell(2, "hexagonal", a0), [A, B], precision)
    sys.add_species(M.Multiblock([A, B], [NA, 100 - NA], [1.0, 1.0], Ns), 1.0)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, chi)
    sys.add_interaction(itx)
    shape = (1, n, n)
    _, y, x = np.meshgrid(np.zeros(1), np.arange(n) / n, np.arange(n) / n, indexing="ij")
    six = amp * (np.cos(2 * np.pi * x) + np.cos(2 * np.pi * y) + np.cos(2 * np.pi * (x + y)))
    M.fieldinit(sys, seeded_fields(shape, [1, 2], seed, scale, six))
    return sys


def bcc_system(M, n=64, L=7.0, precision=None, Ns=100, seed=12345):
    """The 3D BCC workload: AB diblock N100 fA0.30 (built as Multiblock([A, B], [30, 70])),
    chi 0.2, Ns 100, cubic cell L0; w_A = 0.1 N(0,1) + the sum of cos(2 pi h.r / L) over the 12
    {110} reflections (h = (+-1, +-1, 0) and permutations; fractional coordinates on the
    grid) scaled by 1/4 (peak 3; the raw sum peaks at 12, which as a field overflows float64
    propagators at ds = 1, and a peak of 1 decays to the disordered state), w_B = -w_A."""
    A, B = M.Monomer(1), M.Monomer(2)
    sys = _fs(M, (n, n, n), M.UnitCell(3, "cubic", L), [A, B], precision)
    sys.add_species(M.Multiblock([A, B], [30, 70], [1.0, 1.0], Ns), 1.0)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys.add_interaction(itx)
    shape = (n, n, n)
    z, y, x = np.meshgrid(*(np.arange(n) / n for _ in range(3)), indexing="ij")
    pat = np.zeros(shape)
    for a, b in ((x, y), (y, z), (z, x)):  # 6 +-pairs x 2 signs = 12 reflections
        pat += 2.0 * np.cos(2 * np.pi * (a + b)) + 2.0 * np.cos(2 * np.pi * (a - b))
    rng = np.random.Generator(np.random.PCG64(seed))
    wa = 0.1 * rng.standard_normal(shape) + pat / 4.0
    M.fieldinit(sys, {1: wa, 2: -wa})
    return sys


def _julia_seed_fields(case):
    d = np.load(os.path.join(GOLDEN, "julia_seed_fields.npz"))
    pre = f"{case}_w"
    return {int(k[len(pre):]): d[k] for k in d.files if k.startswith(pre)}


def reference_test_system(M, precision=None):
    """test/test_system.jl:3-26: 32x1x1 lamellar (L 10), Point(C) phi 0.75 + Diblock(A, B, N100,
    f0.5, Ns100) phi 0.25, chi_AB 0.2, with the fields of fieldinit!(sys; scale = 0.1,
    seed = 12345) (the Julia randn stream, fixture julia_seed_fields.npz).  Returns
    (sys, point, chain)."""
    A, B, C = M.Monomer(1, 1.0, 0.0), M.Monomer(2, 1.0, 0.0), M.Monomer(3, 1.0, 0.0)
    point = M.Point(C)
    chain = M.Diblock(A, B, 100, 0.5, 1.0, 1.0, 100)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys = _fs(M, (32, 1, 1), M.UnitCell(1, "lamellar", 10.0), [A, B, C], precision)
    sys.add_species(point, 0.75)
    sys.add_species(chain, 0.25)
    sys.add_interaction(itx)
    M.fieldinit(sys, _julia_seed_fields("system"))
    return sys, point, chain


def reference_test_updaters_system(M, precision=None):
    """test/test_updaters.jl:3-14: the same diblock alone (phi 1), same seeded fields."""
    A, B = M.Monomer(1, 1.0, 0.0), M.Monomer(2, 1.0, 0.0)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys = _fs(M, (32, 1, 1), M.UnitCell(1, "lamellar", 10.0), [A, B], precision)
    sys.add_species(M.Diblock(A, B, 100, 0.5, 1.0, 1.0, 100), 1.0)
    sys.add_interaction(itx)
    M.fieldinit(sys, _julia_seed_fields("updaters"))
    return sys


def notebook_blend_seeded_system(M, precision=None):
    """examples/examples.ipynb cell 11: the ABC blend (Point C vol 1 phi 0.4, homopolymers A, B
    vol 2 N100 phi 0.3 each; chi_AB 0.5, chi_AC = chi_BC = 1.25) on 256x1x1 (L 20), with the
    fields of fieldinit!(sys; scale = 0.05, seed = 12345) (fixture julia_seed_fields.npz)."""
    A, B, C = M.Monomer(1, 2.0), M.Monomer(2, 2.0), M.Monomer(3, 1.0)
    sys = _fs(M, (256, 1, 1), M.UnitCell(1, "lamellar", 20.0), [A, B, C], precision)
    sys.add_species(M.Point(C), 0.4)
    sys.add_species(M.Homopolymer(A, 100, 1.0), 0.3)
    sys.add_species(M.Homopolymer(B, 100, 1.0), 0.3)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.5)
    itx.set_interaction(A, C, 1.25)
    itx.set_interaction(B, C, 1.25)
    sys.add_interaction(itx)
    M.fieldinit(sys, _julia_seed_fields("nbblend"))
    return sys
