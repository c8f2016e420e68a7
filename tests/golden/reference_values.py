"""Numbers published by the reference (PolyFields.jl), with the file and line they come from.

These are the parity pins of the oracle and of the GPU engine.  Values printed by the
reference's own runs are copied verbatim; nothing here is computed by this project.
"""
import math

# test/test_cell.jl:3-36 — cell volumes
CELL_VOLUMES = [
    ((1, "lamellar", 10.0), 10.0),
    ((2, "square", 10.0), 100.0),
    ((2, "rectangular", 10.0, 5.0), 50.0),
    ((2, "hexagonal", 10.0), 86.60254037844385),
    ((2, "oblique", 10.0, 5.0, math.pi / 4), 35.35533905932737),
    ((3, "cubic", 10.0), 1000.0),
    ((3, "tetragonal", 10.0, 5.0), 500.0),
    ((3, "orthorhombic", 10.0, 5.0, 2.0), 100.0),
    ((3, "hexagonal", 10.0, 5.0), 433.01270189221924),
    ((3, "monoclinic", 10.0, 5.0, 2.0, math.pi / 4), 70.71067811865474),
    ((3, "triclinic", 10.0, 5.0, 2.0, math.pi / 2, math.pi / 2, math.pi / 2), 100.0),
]

# test/test_species.jl:5-16
SPECIES = {
    "point_Nref": 2.0,             # Point(Monomer(vol=2)).Nref
    "homopolymer_Nref": 100.0,     # Homopolymer(bmon, 100, 1.0, 200).Nref
    "diblock_f_block_1": 0.4,      # Diblock(amon(vol 2), bmon, 100, 0.25, ...).f_block[1]
    "diblock_Nref_block_2": 75.0,  # ... .Nref_block[2]
    "multiblock_fraction_1": 2 / 3,
}

# README.md:62-79 — scft! on 64x1x1 lamellar, Diblock N100 f0.5 Ns100, chi 0.2, Anderson
# nhist 10, DomainUpdater nskip 5 / nper 20, ftol = stol = 1e-4.  Converged state:
README_LAMELLAR = {
    "L": 16.528709413909947,
    "fhelm": 0.0812381288285528,
    "ferr": 5.0874415525661515e-6,
    "serr": 1.6582423877606872e-6,
    "nsteps": 36,
}

# examples/examples.ipynb cell 12 output: ABC blend (Point C vol 1 phi 0.4, homopolymers
# A, B vol 2 N100 phi 0.3 each; chi_AB 0.5, chi_AC = chi_BC = 1.25) on 256x1x1, L = 20.
# The saved seed examples/seeds/abc_blend_1d.json is that converged state, so residuals!
# + field_error + free_energy on the seed reproduce these to rounding.
BLEND_FINAL = {"ferr": 9.9617272806509e-6, "fhelm": -0.04720567097567993}

# examples/examples.ipynb cell 8 output: 128x128 hexagonal cylinders, Diblock N100 f0.3
# Ns100, chi 0.3, cell a = 18.381681210100236 (seed examples/seeds/cyl2d.json is 64x64).
CYL2D_FINAL_128 = {"ferr": 9.910317272221094e-6, "fhelm": 0.10659231121049459,
                   "a": 18.381681210100236}

# examples/examples.ipynb cell 4 output: 128x1x1 lamellar, Diblock N100 f0.5 Ns100, chi
# 0.25, L = 13.100000015310233 (seed examples/seeds/lam1d.json is 64x1x1); converged at
# step 0.
LAM1D_FINAL_128 = {"ferr": 9.713161299981836e-6, "fhelm": 0.10211268214323928}

# test/test_system.jl:3-34 — 32x1x1 lamellar (L 10), Point(C) phi 0.75 + Diblock(A, B, N100,
# f0.5, b 1, 1, Ns100) phi 0.25, chi_AB 0.2, fieldinit!(sys; scale = 0.1, seed = 12345), then
# density!(point), density!(chain).  The fields are Julia's seeded randn stream, restated in
# oracle/julia_rng.py (fixture tests/golden/julia_seed_fields.npz, keys system_w*).
TEST_SYSTEM = {
    "point_Q": 1.004177455788938,
    "chain_Q": 8.24300700515971,
    "free_energy": -0.1681580628744596,
    "free_energy_bulk": -0.9686022902416352,
    "scfstress_1": -0.0004272750367130805,
}

# test/test_updaters.jl:3-30 — the same diblock alone (phi 1) with the same fieldinit!; an
# EulerUpdater(:PECE, lam 0.005), a MomentumUpdater(:NAG, lam 0.005) and an
# AndersonUpdater(nhist 5) are all set up first, then each takes 10 steps in that order
# (fixture keys updaters_w*).  free_energy after the Euler steps (:24) and after the
# Anderson steps (:30); the value after the NAG steps is the file's commented-out check (:27).
TEST_UPDATERS = {
    "after_euler": 0.0626842750325202,
    "after_nag_commented_out": 0.06172669754976512,
    "after_anderson": 0.12798422498635653,
}

# examples/examples.ipynb cells 11-12: the ABC blend of BLEND_FINAL on 256x1x1 (L 20) from
# fieldinit!(sys; scale = 0.05, seed = 12345), relaxed by scft!(sys, MomentumUpdater(method =
# :MOM, lam = 0.01); opts = SCFTOptions(nsteps = 5000, nsout = 500, ftol = 1e-5, stol = 5e-5)).
# Printed lines "Step (k / 5000): ferr = %8e, fhelm = %.5e" (the state after k updates) and
# "Converged @ step = 3272: ferr = %8e, fhelm = %.5e" (the state after 3273 updates: the
# loop breaks before incrementing its counter); the SCFTResults it returned are BLEND_FINAL.
NOTEBOOK_BLEND_RUN = {
    "printed": {0: (1.409117e+00, -7.42676e-02), 500: (5.151726e-02, -4.78117e-02),
                1000: (4.316219e-03, -4.73547e-02), 1500: (9.502502e-04, -4.72453e-02),
                2000: (2.516323e-04, -4.72159e-02), 2500: (6.925002e-05, -4.72081e-02),
                3000: (1.963959e-05, -4.72061e-02)},
    "converged_line": (9.986285e-06, -4.72057e-02),
    "nsteps": 3272,
}
