"""scft_batch: many independent scft! runs driven together (phase-diagram sweeps).

Each system runs on its own stream from a pool of host threads; the kernels are the same as
for a single run, so every batched result must equal the result of running that system
alone, and one failing system must not disturb the others.
"""
import numpy as np
import pytest

pf = pytest.importorskip("polyfields")
from polyfields import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu

PARAMS = [dict(n=32, chi=0.22, NA=30, a0=6.5, seed=1), dict(n=48, chi=0.25, NA=35, a0=7.5, seed=2),
          dict(n=32, chi=0.18, NA=45, a0=5.0, seed=3), dict(n=64, chi=0.20, NA=28, a0=8.0, seed=4),
          dict(n=48, chi=0.28, NA=40, a0=6.0, seed=5), dict(n=32, chi=0.15, NA=50, a0=4.5, seed=6)]


def _build(precision):
    systems = [W.hex_instance(pf, precision=precision, **p) for p in PARAMS]
    ups = [pf.AndersonUpdater(nhist=10) for _ in systems]
    doms = [pf.DomainUpdater(nskip=5, nper=20) for _ in systems]
    return systems, ups, doms


def test_batch_equals_individual_runs_fp64():
    opts = pf.SCFTOptions(nsteps=150, ftol=1e-6, stol=1e-6)
    systems, ups, doms = _build("fp64")
    batched = pf.scft_batch(systems, ups, doms, opts, nthreads=3)
    for i, p in enumerate(PARAMS):
        s = W.hex_instance(pf, precision="fp64", **p)
        r = pf.scft(s, pf.AndersonUpdater(nhist=10), domain=pf.DomainUpdater(nskip=5, nper=20), opts=opts)
        assert batched[i].nsteps == r.nsteps
        assert batched[i].converged == r.converged
        assert batched[i].fhelm == pytest.approx(r.fhelm, rel=1e-12, abs=1e-14)
        assert systems[i].cell.params[0] == pytest.approx(s.cell.params[0], rel=1e-12)
        assert np.array_equal(systems[i].fields[1], s.fields[1])


def test_batch_mixed_polish_reaches_fp64_answers():
    """float32 iterations switched to float64 at ferr < 1e-5, polished to ftol = 1e-7 (cells
    held fixed: with the DomainUpdater the reference's iteration diverges for most of these
    instances in either precision): free energies agree with float64-only runs to 1e-8."""
    opts64 = pf.SCFTOptions(nsteps=3000, ftol=1e-7)
    optsm = pf.SCFTOptions(nsteps=3000, ftol=1e-7, mixed_switch_ferr=1e-5)
    s64, u64, _ = _build("fp64")
    sm, um, _ = _build("fp32")
    r64 = pf.scft_batch(s64, u64, None, opts64)
    rm = pf.scft_batch(sm, um, None, optsm)
    for i in range(len(PARAMS)):
        assert r64[i].converged and rm[i].converged, i
        assert rm[i].switch_step >= 0
        assert abs(rm[i].fhelm - r64[i].fhelm) <= 1e-8, (i, rm[i].fhelm, r64[i].fhelm)


def test_batch_reports_a_failing_system_without_disturbing_the_others():
    opts = pf.SCFTOptions(nsteps=40, ftol=1e-12, stol=1e-12)
    systems, ups, doms = _build("fp64")
    w = systems[2].fields[1]
    w[0, 0, 5] = np.nan
    systems[2].fields[1] = w
    res, st = pf.scft_batch(systems, ups, doms, opts, nthreads=4, raise_on_error=False)
    assert st[2] == pf._lib.PF_ENAN
    assert all(st[i] == 0 for i in range(len(PARAMS)) if i != 2)
    assert all(res[i].nsteps == 40 for i in range(len(PARAMS)) if i != 2)
