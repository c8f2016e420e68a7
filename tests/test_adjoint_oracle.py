"""The FP64 CPU reference gradient (oracle/pf_adjoint.py) against central finite differences
of the oracle's density! on small grids: the pin of every GPU gradient test.

L = sum_x (rho_A - target)^2 with a smooth seeded target; derivatives with respect to single
field values, the cell parameters and the block length of A (composition f at fixed contour
step counts).  Central differences with h = 1e-5 in FP64: agreement to 1e-6 relative.
"""
import numpy as np
import pytest

import pf_oracle as O
import pf_adjoint as AD


def build(dims, crystal, params, NA, NB, fields, Ns=40, blend=False):
    A, B = O.Monomer(1, 1.0), O.Monomer(2, 1.0)
    mons = [A, B]
    if blend:
        C = O.Monomer(3, 1.0)
        mons.append(C)
    nd = sum(1 for d in dims if d > 1)
    sys = O.FieldSystem(dims, O.UnitCell(nd, crystal, *params), monomers=mons)
    if blend:
        sys.add_species(O.Multiblock([A, B], [NA, NB], [1.0, 1.2], Ns), 0.6)
        sys.add_species(O.Homopolymer(A, 40, 1.0, Ns), 0.25)
        sys.add_species(O.Point(C), 0.15)
    else:
        sys.add_species(O.Multiblock([A, B], [NA, NB], [1.0, 1.0], Ns), 1.0)
    itx = O.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys.add_interaction(itx)
    for mid, w in fields.items():
        sys.fields[mid] = w.copy()
    sys.density_update()
    return sys


CASES = [
    ("lam1d", (32, 1, 1), "lamellar", [7.0], False),
    ("hex2d", (16, 16, 1), "hexagonal", [6.0], False),
    ("cubic3d", (8, 8, 8), "cubic", [5.0], False),
    ("blend2d", (16, 8, 1), "rectangular", [6.0, 4.0], True),
]


@pytest.mark.parametrize("name,dims,crystal,params,blend", CASES, ids=[c[0] for c in CASES])
def test_pullback_matches_central_differences(name, dims, crystal, params, blend):
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(11)
    mids = [1, 2, 3] if blend else [1, 2]
    fields = {m: 0.4 * rng.standard_normal(shape) for m in mids}
    NA, NB = 35.0, 65.0
    target = AD.smooth_target(shape, 0.35, amp=0.2, nmodes=5, seed=5)

    def loss(fields=fields, params=params, NA=NA, NB=NB):
        s = build(dims, crystal, params, NA, NB, fields, blend=blend)
        return AD.density_loss(s, 1, target)[0]

    sys = build(dims, crystal, params, NA, NB, fields, blend=blend)
    L0, rbar = AD.density_loss(sys, 1, target)
    g = AD.density_pullback(sys, rbar)
    h = 1e-5
    # single field values of every monomer
    for m in mids:
        for flat in rng.choice(int(np.prod(shape)), size=3, replace=False):
            idx = np.unravel_index(flat, shape)
            fp = {k: v.copy() for k, v in fields.items()}
            fm = {k: v.copy() for k, v in fields.items()}
            fp[m][idx] += h
            fm[m][idx] -= h
            fd = (loss(fields=fp) - loss(fields=fm)) / (2 * h)
            assert g["w"][m][idx] == pytest.approx(fd, rel=1e-6, abs=1e-10 * abs(L0)), (m, idx)
    # cell parameters
    for p in range(len(params)):
        pp, pm = list(params), list(params)
        pp[p] += h
        pm[p] -= h
        fd = (loss(params=pp) - loss(params=pm)) / (2 * h)
        assert g["cell"][p] == pytest.approx(fd, rel=1e-6, abs=1e-12), p
    # composition: block A longer, block B shorter (contour step counts unchanged)
    fd = (loss(NA=NA + h, NB=NB - h) - loss(NA=NA - h, NB=NB + h)) / (2 * h)
    dN = g["Nref_block"][0]
    assert dN[0] - dN[1] == pytest.approx(fd, rel=1e-6, abs=1e-12)
    assert all(v == 0.0 for v in g["chi"].values())


def test_simpson_weights_match_the_reference_sum():
    for n in (2, 3, 4, 7, 10):
        w = AD.simpson_weights(n)
        x = np.linspace(0.0, 1.0, n + 1)
        if n % 2 == 0:  # exact for cubics on an even number of intervals
            assert np.dot(w, x ** 3) / 3.0 / n == pytest.approx(0.25, rel=1e-12)
        assert w[0] == 1.0 and w[n] == 1.0


FE_CASES = [
    ("hex2d", (16, 16, 1), "hexagonal", [6.0], False),
    ("cubic3d", (8, 8, 8), "cubic", [5.0], False),
    ("blend2d", (16, 8, 1), "rectangular", [6.0, 4.0], True),
]


@pytest.mark.parametrize("name,dims,crystal,params,blend", FE_CASES, ids=[c[0] for c in FE_CASES])
def test_free_energy_pullback_matches_central_differences(name, dims, crystal, params, blend):
    """d free_energy / d(w, cell, N_A, chi) at fixed fields (src/system/system.jl:402-433) against
    central differences of the oracle's free_energy."""
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(17)
    mids = [1, 2, 3] if blend else [1, 2]
    fields = {m: 0.4 * rng.standard_normal(shape) for m in mids}
    NA, NB = 35.0, 65.0

    def fhelm(fields=fields, params=params, NA=NA, chi=0.2):
        s = build(dims, crystal, params, NA, NB, fields, blend=blend)
        s.interactions[0].chis[(1, 2)] = chi
        return s.free_energy()

    sys = build(dims, crystal, params, NA, NB, fields, blend=blend)
    g = AD.free_energy_pullback(sys)
    h = 1e-5

    def cd(f):
        return (f(+h) - f(-h)) / (2 * h)

    for m in mids:
        for idx in [(0, 0, 3), (shape[0] - 1, shape[1] - 1, shape[2] - 2)]:
            def fw(d, m=m, idx=idx):
                f2 = {k: v.copy() for k, v in fields.items()}
                f2[m][idx] += d
                return fhelm(fields=f2)
            assert g["w"][m][idx] == pytest.approx(cd(fw), rel=1e-6, abs=1e-12), (m, idx)
    for p in range(len(params)):
        def fc(d, p=p):
            q = list(params)
            q[p] += d
            return fhelm(params=q)
        assert g["cell"][p] == pytest.approx(cd(fc), rel=1e-6, abs=1e-12)
    assert g["Nref_block"][0][0] == pytest.approx(cd(lambda d: fhelm(NA=NA + d)), rel=1e-6, abs=1e-12)
    assert g["chi"][(1, 2)] == pytest.approx(cd(lambda d: fhelm(chi=0.2 + d)), rel=1e-7)
    assert g["chi"][(1, 2)] != 0.0
