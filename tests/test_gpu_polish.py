"""Float64 polish of the mixed-precision scft!: Newton-Krylov steps with float32 Jacobian
products reach the plain float64 solver's fixed point (src/simulate.jl:60-148 run to ftol).

The 3D blend (AB diblock N100 fA0.4 phi0.8 + A homopolymer N50, Ns 200, cubic L 14, double
gyroid start) at 32^3 with the cell held fixed: the float64 run and both mixed variants must
converge to ftol = 1e-8 with |dfhelm| <= 1e-8, and the Newton polish must need far fewer
float64 density solves than float64 Anderson steps after the switch.  The Newton polish is
checked from a late switch (ferr 3e-6) and from an early one (3e-3, as bench.py's time-to-solution
runs use), where it replaces most of the float32 Anderson iterations.
"""
import pytest

from polyfields import workloads as W

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fp64_answer():
    s = W.blend3d_system(pf, n=32, precision="fp64")
    r = pf.scft(s, pf.AndersonUpdater(nhist=20), opts=pf.SCFTOptions(nsteps=4000, ftol=1e-8))
    assert r.converged
    return r


def _mixed(polish, switch=3e-6):
    s = W.blend3d_system(pf, n=32, precision="fp32")
    opts = pf.SCFTOptions(nsteps=4000, ftol=1e-8, mixed_switch_ferr=switch, polish=polish)
    return pf.scft(s, pf.AndersonUpdater(nhist=20), opts=opts), s


@pytest.mark.parametrize("switch", [3e-6, 3e-3])
def test_newton_polish_reaches_the_fp64_fixed_point(fp64_answer, switch):
    r, s = _mixed("newton", switch)
    assert r.converged and r.switch_step >= 0
    assert r.ferr < 1e-8 and s.field_error() < 1e-8
    assert abs(r.fhelm - fp64_answer.fhelm) <= 1e-8
    assert 2 <= r.polish_fp64_solves <= 12
    assert r.polish_fp32_solves > 0


def test_updater_polish_reaches_the_fp64_fixed_point(fp64_answer):
    r, _ = _mixed("updater")
    assert r.converged and r.switch_step >= 0
    assert abs(r.fhelm - fp64_answer.fhelm) <= 1e-8
    assert r.polish_fp64_solves == 0 and r.polish_fp32_solves == 0
    assert r.nsteps - r.switch_step > 20  # float64 Anderson steps after the switch
