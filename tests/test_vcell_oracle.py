"""The DomainUpdater (src/updaters/domain.jl:50-121) on sweep instances, in the FP64 oracle.

With the reference's defaults (lam 0.1, pmax 1, rlxn 0.5, finite-difference Jacobian with
dx = 1e-8) and AndersonUpdater(nhist = 10), nskip 5, nper 20, the reference's own iteration
runs away on this 2D hexagonal diblock instance of the phase-diagram sweep (32^2, chiN 15.1,
N_A 31, a0 7.42): every cell update moves the cell by the step cap until the propagators
overflow and scft! stops with "Diverging field updater -- breaking." (src/simulate.jl:109-111).
The GPU engine does the same (tests/test_gpu_vcell.py); it is the algorithm's behaviour on
this system, not an effect of precision.
"""
import numpy as np
import pytest

import pf_oracle as O
from polyfields import workloads as W

INSTANCE = dict(n=32, chi=0.15138733956444989, NA=31, a0=7.424114923196996, seed=1362635735)


def test_oracle_domain_updater_runs_away_and_diverges():
    s = W.hex_instance(O, **INSTANCE)
    d = O.DomainUpdater(nskip=5, nper=20)
    cells = []
    orig = d.step

    def rec(*a, **k):
        r = orig(*a, **k)
        cells.append(float(s.cell.params[0]))
        return r

    d.step = rec
    with np.errstate(all="ignore"), pytest.raises(RuntimeError, match="Diverging field updater"):
        O.scft(s, O.AndersonUpdater(nhist=10), domain=d, opts=O.SCFTOptions(nsteps=400, ftol=1e-7, stol=1e-7))
    # the first two updates each move a0 by about nper * rlxn * lam * pmax = 0.95
    assert cells[0] == pytest.approx(INSTANCE["a0"] + 0.95, abs=1e-6)
    assert cells[1] == pytest.approx(INSTANCE["a0"] + 1.90, abs=1e-6)
