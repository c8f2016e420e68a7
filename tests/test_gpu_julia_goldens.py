"""The reference's RNG-dependent test goldens on the GPU engine (through the C ABI).

Same systems and fields as tests/test_julia_seed_goldens.py (test/test_system.jl,
test/test_updaters.jl with Julia's seeded randn stream, fixture julia_seed_fields.npz).  The
float64 engine must give the reference's asserted numbers at the float64 parity bar.  The
updater sequence also checks that updaters set up on one system keep separate state: the Euler
updater steps correctly after the NAG and Anderson updaters were created on the same system.
"""
import math

import pytest

import pf_oracle as O
import reference_values as RV
from polyfields import workloads as W

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10


def _system(precision):
    """The test's system after `fieldinit!` and its `density!(point); density!(chain)`
    (test/test_system.jl:23-27): the second solve runs on the fields that residuals! inside
    fieldinit! mean-subtracted, and the goldens come from it."""
    sys, point, chain = W.reference_test_system(pf, precision=precision)
    sys.density_update()
    return sys, point, chain


def test_test_system_goldens_fp64():
    sys, point, chain = _system("fp64")
    g = RV.TEST_SYSTEM
    assert point.Q == pytest.approx(g["point_Q"], rel=FP64_RTOL)
    assert chain.Q == pytest.approx(g["chain_Q"], rel=FP64_RTOL)
    assert sys.free_energy() == pytest.approx(g["free_energy"], rel=FP64_RTOL)
    assert sys.free_energy_bulk() == pytest.approx(g["free_energy_bulk"], rel=FP64_RTOL)
    assert sys.scfstress()[0] == pytest.approx(g["scfstress_1"], rel=1e-9)


def test_test_system_goldens_fp32():
    """Float32 chains (float64 reductions): Q to the float32 parity bar, the free energy and
    the stress to what float32 propagators carry."""
    sys, point, chain = _system("fp32")
    g = RV.TEST_SYSTEM
    assert point.Q == pytest.approx(g["point_Q"], rel=5e-5)
    assert chain.Q == pytest.approx(g["chain_Q"], rel=5e-5)
    assert sys.free_energy() == pytest.approx(g["free_energy"], rel=1e-4)
    assert sys.free_energy_bulk() == pytest.approx(g["free_energy_bulk"], rel=1e-12)
    assert sys.scfstress()[0] == pytest.approx(g["scfstress_1"], rel=1e-2)


def test_test_updaters_goldens_fp64():
    g = RV.TEST_UPDATERS
    s = W.reference_test_updaters_system(pf, precision="fp64")
    o = W.reference_test_updaters_system(O)
    ug = [pf.EulerUpdater(method="PECE", lam=0.005), pf.MomentumUpdater(method="NAG", lam=0.005),
          pf.AndersonUpdater(nhist=5)]
    uo = [O.EulerUpdater(method="PECE", lam=0.005), O.MomentumUpdater(method="NAG", lam=0.005),
          O.AndersonUpdater(nhist=5)]
    for a, b in zip(ug, uo):
        a.setup(s)
        b.setup(o)
    expect = [g["after_euler"], g["after_nag_commented_out"], g["after_anderson"]]
    tol = [FP64_RTOL, FP64_RTOL, math.sqrt(2.220446049250313e-16)]  # Anderson: the reference test's isapprox
    for k in range(3):
        for _ in range(10):
            ug[k].step()
            uo[k].step()
        assert s.free_energy() == pytest.approx(expect[k], rel=tol[k]), k
        assert s.free_energy() == pytest.approx(o.free_energy(), rel=1e-8 if k == 2 else FP64_RTOL), k
    # back to the first updater after the others ran on the same system
    ug[0].step()
    uo[0].step()
    assert s.free_energy() == pytest.approx(o.free_energy(), rel=1e-8)


def test_seeded_fieldinit_as_the_reference_test_writes_it():
    """test/test_system.jl:3-33 line for line through the Python mirror: its own seeded
    fieldinit (Julia's stream, polyfields.julia_random) instead of the fixture."""
    amon = pf.Monomer(1, 1.0, 0.0)
    bmon = pf.Monomer(2, 1.0, 0.0)
    cmon = pf.Monomer(3, 1.0, 0.0)
    point = pf.Point(cmon)
    chain = pf.Diblock(amon, bmon, 100, 0.5, 1.0, 1.0, 100)
    itx = pf.FloryInteraction()
    itx.set_interaction(amon, bmon, 0.2)
    sys = pf.FieldSystem((32, 1, 1), pf.UnitCell(1, "lamellar", 10.0), monomers=[amon, bmon, cmon],
                         precision="fp64")
    sys.add_species(point, 0.75)
    sys.add_species(chain, 0.25)
    sys.add_interaction(itx)
    pf.fieldinit(sys, scale=0.1, seed=12345)
    sys.density_update()
    g = RV.TEST_SYSTEM
    assert point.Q == pytest.approx(g["point_Q"], rel=FP64_RTOL)
    assert chain.Q == pytest.approx(g["chain_Q"], rel=FP64_RTOL)
    assert sys.free_energy() == pytest.approx(g["free_energy"], rel=FP64_RTOL)
    assert sys.scfstress()[0] == pytest.approx(g["scfstress_1"], rel=1e-9)
