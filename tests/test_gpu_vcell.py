"""Variable cell (DomainUpdater, src/updaters/domain.jl:50-121) on the GPU against the oracle.

1. A sweep instance on which the reference's iteration runs away (tests/test_vcell_oracle.py):
   the GPU's cell after each of the first two cell updates equals the oracle's to 1e-6 (the
   finite-difference Jacobian, dx = 1e-8, amplifies rounding differences of the stress), and
   scft! on the GPU stops with the same error.
2. Cases that converge with the cell free.  The reference's stress sums Re(q_k) Re(qc_k)
   (src/species/multiblock.jl:279-282), not Re(q_k conj(qc_k)), so it depends on where the
   structure sits in the box: a structure translated along a zero mode of the field iteration
   has its zero stress at another cell (tests/test_vcell_oracle.py).  From a noisy start the
   two precisions drift apart along that mode and converged 0.8% apart in the cell (so do two
   float64 runs from different noise); a start with mirror symmetry keeps the structure in
   place, its spectra real and the converged cell unique.  So the cases are the README lamellar system
   (config 1: 64 x 1 x 1, chi 0.2, Anderson nhist 10, DomainUpdater nskip 5, nper 20) from a
   cosine start at L = 13, and the notebook's hexagonal cylinder seed (examples/seeds/cyl2d.json,
   64^2, with its own settings MomentumUpdater MOM lam 0.1, DomainUpdater nskip 100, nper 10).
   For the cylinders, float64 throughout and the mixed path (float32 iterations, whose cell
   updates use a finite-difference step of 1e-4, then float64) run to tight ftol/stol reach
   the same cell within 1e-6 and the same free energy within 1e-8.  For the lamellae the
   float64 run matches the oracle's to those tolerances, and the mixed run's answer is a fixed
   point of the float64 reference iteration, with the lamella moved slightly along the zero
   mode by the float32 phase (test docstring).
"""
import numpy as np
import pytest

import pf_oracle as O
import systems as SY
from polyfields import workloads as W

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu

INSTANCE = dict(n=32, chi=0.15138733956444989, NA=31, a0=7.424114923196996, seed=1362635735)


def test_runaway_cell_tracks_the_oracle_and_diverges():
    o = W.hex_instance(O, **INSTANCE)
    g = W.hex_instance(pf, precision="fp64", **INSTANCE)
    uo, ug = O.AndersonUpdater(nhist=10), pf.AndersonUpdater(nhist=10)
    do, dg = O.DomainUpdater(nskip=5, nper=20), pf.DomainUpdater(nskip=5, nper=20)
    uo.setup(o)
    ug.setup(g)
    do.setup(o)
    dg.setup(g)
    for step in range(6):  # scft!'s loop (simulate.jl:86-103) up to the second cell update
        uo.step()
        ug.step()
        if step % 5 == 0:
            do.step(nsteps=20)
            dg.step(nsteps=20)
            assert float(g.cell.params[0]) == pytest.approx(float(o.cell.params[0]), rel=1e-6), step
    h = W.hex_instance(pf, precision="fp64", **INSTANCE)
    with pytest.raises(pf.PolyFieldsError, match="Diverging field updater"):
        pf.scft(h, pf.AndersonUpdater(nhist=10), domain=pf.DomainUpdater(nskip=5, nper=20),
                opts=pf.SCFTOptions(nsteps=400, ftol=1e-7, stol=1e-7))


def test_bcc_cell_trajectory_tracks_the_oracle():
    """The BCC workload (AB diblock fA 0.3, chi 0.2, cubic L0 = 7, the 12 {110} cosines plus 0.1
    noise) at 16^3 with Anderson nhist 10 and DomainUpdater nskip 5 / nper 20, float64: through
    the first 30 iterations of scft!'s loop (simulate.jl:86-103, six cell updates) the GPU's cell
    after every update equals the oracle's to 1e-6.  The reference's cell steps back and forth
    by the step cap (nper rlxn lam pmax = 0.95) and then walks away from 7 (the oracle, run on,
    leaves it near 15 after 300 iterations without converging): it is the reference iteration,
    not the GPU, that does not settle this cell."""
    o = W.bcc_system(O, n=16)
    g = W.bcc_system(pf, n=16, precision="fp64")
    uo, ug = O.AndersonUpdater(nhist=10), pf.AndersonUpdater(nhist=10)
    do, dg = O.DomainUpdater(nskip=5, nper=20), pf.DomainUpdater(nskip=5, nper=20)
    uo.setup(o)
    ug.setup(g)
    do.setup(o)
    dg.setup(g)
    cells = []
    for step in range(30):
        uo.step()
        ug.step()
        if step % 5 == 0:
            do.step(nsteps=20)
            dg.step(nsteps=20)
            cells.append(float(o.cell.params[0]))
            assert float(g.cell.params[0]) == pytest.approx(cells[-1], rel=1e-6), step
    assert cells[0] == pytest.approx(7.95, abs=1e-6) and cells[1] == pytest.approx(8.90, abs=1e-6)
    assert cells[-1] > 10.0


def _mixed_vs_fp64(make, updater, domain, ftol, stol, nsteps):
    g64 = make("fp64")
    r64 = pf.scft(g64, updater(), domain=domain(), opts=pf.SCFTOptions(nsteps=nsteps, ftol=ftol, stol=stol))
    gm = make("fp32")
    rm = pf.scft(gm, updater(), domain=domain(),
                 opts=pf.SCFTOptions(nsteps=nsteps, ftol=ftol, stol=stol, mixed_switch_ferr=1e-5))
    print("variable cell:", r64, rm, g64.cell.params, gm.cell.params)
    assert r64.converged and rm.converged
    assert rm.switch_step >= 0
    assert np.allclose(gm.cell.params, g64.cell.params, rtol=1e-6, atol=0)
    assert abs(rm.fhelm - r64.fhelm) <= 1e-8
    return g64, r64


def _oracle_settle(o):
    """Oracle scft! (Anderson nhist 10, DomainUpdater nskip 5 / nper 20, ftol = stol = 1e-9),
    called again until a call converges at entry, where the stress is computed afresh."""
    for _ in range(6):
        r = O.scft(o, O.AndersonUpdater(nhist=10), domain=O.DomainUpdater(nskip=5, nper=20),
                   opts=O.SCFTOptions(nsteps=3000, ftol=1e-9, stol=1e-9))
        assert r.converged
        if r.nsteps == 0:
            return r
    raise AssertionError("no call converged at entry")


def test_variable_cell_lamellar_against_the_oracle():
    """README lamellar system from a cosine start at L = 13.  Float64 on the GPU lands on the
    oracle's cell (1e-6) and free energy (1e-8).  The mixed run (float32 to ferr 1e-5, then
    float64 to ftol = stol = 1e-9) ends on a fixed point of the float64 reference iteration:
    the oracle started from its fields and cell settles there (cell 1e-6, free energy 1e-8).
    Its float32 phase moved the lamella off the mirror-symmetric position (the field
    iteration's zero mode; measured 3.3e-6 relative in the cell), and the reference's stress
    moves the cell with the structure, so the mixed cell is held to the float64 one at 1e-5."""
    kw = dict(dims=(64, 1, 1), crystal="lamellar", params=(13.0,), scale=0.0, amp=0.5)
    opts = dict(nsteps=3000, ftol=1e-9, stol=1e-9)
    g64 = SY.diblock_system(pf, precision="fp64", **kw)
    r64 = pf.scft(g64, pf.AndersonUpdater(nhist=10), domain=pf.DomainUpdater(nskip=5, nper=20),
                  opts=pf.SCFTOptions(**opts))
    o = SY.diblock_system(O, **kw)
    ro = O.scft(o, O.AndersonUpdater(nhist=10), domain=O.DomainUpdater(nskip=5, nper=20),
                opts=O.SCFTOptions(**opts))
    assert r64.converged and ro.converged
    assert np.allclose(g64.cell.params, o.cell.params, rtol=1e-6, atol=0)
    assert abs(r64.fhelm - ro.fhelm) <= 1e-8
    gm = SY.diblock_system(pf, precision="fp32", **kw)
    rm = pf.scft(gm, pf.AndersonUpdater(nhist=10), domain=pf.DomainUpdater(nskip=5, nper=20),
                 opts=pf.SCFTOptions(mixed_switch_ferr=1e-5, **opts))
    print("lamellar:", r64, rm, g64.cell.params, gm.cell.params)
    assert rm.converged and rm.switch_step >= 0
    o2 = SY.diblock_system(O, **dict(kw, params=tuple(float(v) for v in gm.cell.params)))
    O.fieldinit(o2, {m: np.array(gm.fields[m]) for m in (1, 2)})
    r2 = _oracle_settle(o2)
    assert np.allclose(o2.cell.params, gm.cell.params, rtol=1e-6, atol=0)
    assert abs(r2.fhelm - rm.fhelm) <= 1e-8
    assert np.allclose(gm.cell.params, g64.cell.params, rtol=1e-5, atol=0)


def test_variable_cell_mixed_reaches_the_fp64_cell_cylinders():
    _mixed_vs_fp64(lambda prec: SY.cyl2d_seed_system(pf, precision=prec),
                   lambda: pf.MomentumUpdater(method="MOM", lam=0.1), lambda: pf.DomainUpdater(nskip=100, nper=10),
                   1e-8, 1e-9, 12000)
