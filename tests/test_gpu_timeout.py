"""Bounded device waits of the 3D pencil pass: a wait that runs out is reported, per handle.

The pencil pass (z_pipe_kernel) waits on an mbarrier for the TMA copies of each tile with a
time limit (1 s of GPU time by default).  A wait that gives up writes the launch's owner's
status word, drains the copies already in flight (default limit) and exits; the next call that
reads results returns PF_ETIMEOUT and the handle stays usable.  Here the limit is set to zero,
so every such wait gives up at once: no GPU fault, hang or trap is involved.
"""
import numpy as np
import pytest

import pf_oracle as O
import systems as SY

pf = pytest.importorskip("polyfields")
from polyfields import _lib as L  # noqa: E402

pytestmark = pytest.mark.gpu

KW = dict(dims=(16, 16, 16), crystal="cubic", params=(6.0,), f=0.3, amp=0.15)
TOL = {"fp64": 1e-10, "fp32": 5e-5}


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_pencil_wait_timeout_is_reported_and_the_handle_recovers(prec):
    o = SY.diblock_system(O, **KW)
    o.density_update()  # at the mean-subtracted fields that fieldinit leaves, as the GPU solves below
    g = SY.diblock_system(pf, precision=prec, **KW)
    g.set_wait_limit(0.0)
    g.density_update()
    with pytest.raises(pf.PolyFieldsError) as err:
        g.free_energy()
    assert err.value.status == L.PF_ETIMEOUT
    assert "time limit" in str(err.value)
    # the status was read and cleared; with the default limit the next solve is valid
    g.set_wait_limit(1.0)
    g.density_update()
    assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=TOL[prec])
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < TOL[prec]


def test_timeout_of_one_batched_system_does_not_leak_into_the_others():
    """pf_scft_batch runs systems concurrently on their own streams: the system whose pencil
    waits run out fails with PF_ETIMEOUT, the others match their one-at-a-time runs."""
    opts = pf.SCFTOptions(nsteps=30, ftol=1e-12)
    seeds = (3, 4, 5)

    def build(seed):
        return SY.diblock_system(pf, precision="fp64", seed=seed, **KW)

    systems = [build(s) for s in seeds]
    systems[1].set_wait_limit(0.0)
    res, st = pf.scft_batch(systems, [pf.AndersonUpdater(nhist=5) for _ in systems], None, opts, nthreads=3,
                            raise_on_error=False)
    assert st[1] == L.PF_ETIMEOUT
    for i in (0, 2):
        assert st[i] == L.PF_OK
        alone = build(seeds[i])
        r = pf.scft(alone, pf.AndersonUpdater(nhist=5), opts=opts)
        assert res[i].nsteps == r.nsteps
        assert res[i].fhelm == pytest.approx(r.fhelm, rel=1e-12)
        assert np.array_equal(systems[i].fields[1], alone.fields[1])
    # the failed handle is still usable once the limit is back to the default
    systems[1].set_wait_limit(1.0)
    systems[1].density_update()
    assert np.isfinite(systems[1].free_energy())
