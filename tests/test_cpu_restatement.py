"""The C++/OpenMP FP64 CPU restatement (oracle/pf_cpu.cpp) against the NumPy oracle.

Both restate the same reference functions (src/system/mde.jl, src/species/multiblock.jl,
src/system/system.jl, src/interactions/flory.jl, src/system/compress.jl,
src/updaters/anderson.jl); the C++ one, with its own mixed-radix FFT, is bench.py's timed CPU
baseline.  Propagators, densities, residuals, free energy and field error agree to 1e-12
relative; ten Anderson steps (whose small least-squares solve amplifies rounding) to 1e-9.
The restatement also reproduces the reference's own test/test_system.jl goldens.
"""
import numpy as np
import pytest

import pf_cpu as C
import pf_oracle as O
import systems as SY
from polyfields import workloads as W


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b)) / np.max(np.abs(b)))


PROP = [((64, 1, 1), "lamellar", (10.0,)), ((96, 1, 1), "lamellar", (10.0,)), ((32, 32, 1), "hexagonal", (9.0,)),
        ((64, 32, 1), "rectangular", (12.0, 7.0)), ((16, 16, 16), "cubic", (6.0,)), ((48, 48, 48), "cubic", (8.0,)),
        ((32, 16, 8), "orthorhombic", (7.0, 5.0, 4.0)),
        # odd row counts (a last row without a partner) and partial batches of row pairs
        ((24, 9, 1), "rectangular", (8.0, 5.0)), ((18, 18, 3), "orthorhombic", (6.0, 6.0, 2.0)),
        ((36, 27, 9), "orthorhombic", (7.0, 6.0, 3.0))]


@pytest.mark.parametrize("dims,crystal,params", PROP, ids=["x".join(map(str, p[0])) for p in PROP])
def test_propagate_matches_oracle(dims, crystal, params):
    nd = sum(1 for d in dims if d > 1)
    cell = O.UnitCell(nd, crystal, *params)
    cell.setup(dims)
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(3)
    w = 0.3 * rng.standard_normal(shape)
    q0 = 1.0 + 0.1 * rng.standard_normal(shape)
    s = O.PseudoSpectralSolver(dims)
    s.update(w, cell.ksq, 1.3, 1.1, 0.5)
    q, out = q0.copy(), np.empty(shape)
    for _ in range(5):
        s.propagate(q, out)
        q = out.copy()
    got = C.CpuSystem(dims, cell.ksq).propagate(w, 1.3, 1.1, 0.5, q0, 5)
    assert rel(got, q) < 1e-12


SYSTEMS = [("blend3d_16", lambda M: W.blend3d_system(M, n=16)),
           ("hex2d_32", lambda M: SY.diblock_system(M, dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), f=0.3,
                                                    chi=0.3)),
           ("blend_seed_1d", lambda M: SY.blend_seed_system(M))]


@pytest.mark.parametrize("name,make", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_iteration_matches_oracle(name, make):
    """residuals! + free_energy + field_error at the injected fields, then ten Anderson steps."""
    o = make(O)
    c = C.CpuSystem.from_oracle(o)
    o.residuals_update()  # at the mean-subtracted fields that fieldinit leaves, as c starts from
    c.residuals()
    for isp, sp in enumerate(o.species):
        assert c.species_q(isp) == pytest.approx(sp.Q, rel=1e-12)
    for mid in o.monomers:
        assert rel(c.density(mid), o.density[mid]) < 1e-12
        assert np.max(np.abs(c.residuals_grid(mid) - o.residuals[mid])) < 1e-12 * np.max(np.abs(o.fields[mid]))
    assert c.free_energy() == pytest.approx(o.free_energy(), rel=1e-12)
    assert c.field_error() == pytest.approx(o.field_error(), rel=1e-9, abs=1e-15)
    uo = O.AndersonUpdater(nhist=4)
    uo.setup(o)
    c.anderson_setup(4)
    for _ in range(10):
        uo.step()
        c.anderson_step()
    for mid in o.monomers:
        assert rel(c.fields(mid), o.fields[mid]) < 1e-9


def test_uses_several_threads():
    c = C.CpuSystem((16, 1, 1), np.zeros((1, 1, 9)))
    assert c.threads >= 1


def test_reproduces_the_reference_test_system_goldens():
    """test/test_system.jl:29-33 on the C++ restatement itself (the timed reference arm): the
    seeded fields of fieldinit! (Julia's randn stream, fixture julia_seed_fields.npz), then
    density! of each species and free_energy."""
    import reference_values as RV
    o, _, _ = W.reference_test_system(O)
    c = C.CpuSystem.from_oracle(o)
    c.residuals()  # density! at the fields fieldinit! left (mean-subtracted)
    g = RV.TEST_SYSTEM
    assert c.species_q(0) == pytest.approx(g["point_Q"], rel=1e-13)
    assert c.species_q(1) == pytest.approx(g["chain_Q"], rel=1e-13)
    assert c.free_energy() == pytest.approx(g["free_energy"], rel=1e-13)
