"""GPU pullback of density! against the FP64 CPU reference gradient (oracle/pf_adjoint.py,
itself pinned to central finite differences in test_adjoint_oracle.py).

L = sum_x (rho_A - target)^2 with a smooth seeded target.  FP64 chains: dL/dw, dL/dtheta
and dL/dNref_b to 1e-9 relative (of each gradient's largest entry).  FP32 chains (rescaled
histories, FP64 accumulation): 1e-3 relative, float32 rounding over ~80 forward and
adjoint steps.
"""
import numpy as np
import pytest

import pf_oracle as O
import pf_adjoint as AD

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu


def build(M, dims, crystal, params, fields, blend=False, precision=None, Ns=40):
    A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
    mons = [A, B] + ([M.Monomer(3, 1.0)] if blend else [])
    nd = sum(1 for d in dims if d > 1)
    cell = M.UnitCell(nd, crystal, *params)
    sys = M.FieldSystem(dims, cell, monomers=mons) if precision is None else \
        M.FieldSystem(dims, cell, monomers=mons, precision=precision)
    if blend:
        sys.add_species(M.Multiblock([A, B], [35, 65], [1.0, 1.2], Ns), 0.6)
        sys.add_species(M.Homopolymer(A, 40, 1.0, Ns), 0.25)
        sys.add_species(M.Point(mons[2]), 0.15)
    else:
        sys.add_species(M.Multiblock([A, B], [35, 65], [1.0, 1.0], Ns), 1.0)
    itx = M.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys.add_interaction(itx)
    if M is O:
        for mid, w in fields.items():
            sys.fields[mid] = w.copy()
    else:
        for mid, w in fields.items():
            sys.fields[mid] = w
    return sys


CASES = [
    ("lam1d", (32, 1, 1), "lamellar", [7.0], False),
    ("hex2d", (32, 32, 1), "hexagonal", [6.0], False),
    ("rect2d_blend", (32, 16, 1), "rectangular", [6.0, 4.0], True),
    ("cubic3d", (16, 16, 16), "cubic", [5.0], False),
    ("cubic3d_blend", (32, 32, 32), "cubic", [7.0], True),
]


def relmax(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-3)])
@pytest.mark.parametrize("name,dims,crystal,params,blend", CASES, ids=[c[0] for c in CASES])
def test_pullback_matches_reference_gradient(name, dims, crystal, params, blend, prec, tol):
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(21)
    mids = [1, 2, 3] if blend else [1, 2]
    fields = {m: 0.4 * rng.standard_normal(shape) for m in mids}
    target = AD.smooth_target(shape, 0.35, amp=0.2, nmodes=5, seed=5)
    o = build(O, dims, crystal, params, fields, blend)
    o.density_update()
    _, rbar = AD.density_loss(o, 1, target)
    go = AD.density_pullback(o, rbar)
    g = build(pf, dims, crystal, params, fields, blend, precision=prec)
    gg = g.density_pullback(rbar)
    for m in mids:
        assert relmax(gg["w"][m], go["w"][m]) < tol, (m, relmax(gg["w"][m], go["w"][m]))
    assert relmax(gg["cell"], go["cell"]) < tol
    for a, b in zip(gg["Nref_block"], go["Nref_block"]):
        if b:
            assert relmax(a, b) < tol
    assert all(v == 0.0 for v in gg["chi"].values())


def test_pullback_is_linear_in_the_cotangent():
    """pullback(a r1 + b r2) = a pullback(r1) + b pullback(r2) (FP64, 3D)."""
    dims, shape = (16, 16, 16), (16, 16, 16)
    rng = np.random.default_rng(4)
    fields = {m: 0.3 * rng.standard_normal(shape) for m in (1, 2)}
    g = build(pf, dims, "cubic", [5.0], fields, precision="fp64")
    r1 = {1: rng.standard_normal(shape)}
    r2 = {1: rng.standard_normal(shape), 2: rng.standard_normal(shape)}
    p1, p2 = g.density_pullback(r1), g.density_pullback(r2)
    p3 = g.density_pullback({1: 2.0 * r1[1] - 0.5 * r2[1], 2: -0.5 * r2[2]})
    for m in (1, 2):
        assert relmax(p3["w"][m], 2.0 * p1["w"][m] - 0.5 * p2["w"][m]) < 1e-10
    assert relmax(p3["cell"], 2.0 * p1["cell"] - 0.5 * p2["cell"]) < 1e-10
