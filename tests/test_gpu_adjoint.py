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


def test_torch_autograd_density_matches_pullback():
    """polyfields.autodiff.density as a torch op: backward of sum((rho_A - t)^2) equals the
    pullback with rho_bar = 2 (rho_A - t)."""
    torch = pytest.importorskip("torch")
    from polyfields import autodiff
    dims, shape = (32, 32, 1), (1, 32, 32)
    rng = np.random.default_rng(8)
    fields = {m: 0.3 * rng.standard_normal(shape) for m in (1, 2)}
    g = build(pf, dims, "hexagonal", [6.0], fields, precision="fp64")
    target = torch.from_numpy(AD.smooth_target(shape, 0.35, seed=9))
    wt = {m: torch.from_numpy(fields[m]).requires_grad_(True) for m in (1, 2)}
    rho = autodiff.density(g, wt)
    loss = torch.sum((rho[1] - target) ** 2)
    loss.backward()
    pb = g.density_pullback({1: 2.0 * (rho[1].detach().numpy() - target.numpy())})
    for m in (1, 2):
        assert relmax(wt[m].grad.numpy(), pb["w"][m]) < 1e-12


def test_adjoint_96cubed_against_reference_gradient_and_differences():
    """The differentiation workload: 96^3 cubic cell L = 8, AB diblock N = 100, fA = 0.35,
    Ns = 200, chi = 0.2, propagators recomputed between checkpoints every 15 contour steps;
    L = sum (rho_A - target)^2 with a smooth seeded target (5 lowest modes, amplitude 0.2,
    mean fA).  GPU FP64 vs the FP64 CPU reference gradient (1e-9),
    GPU FP32 chains vs the same (1e-3), and central differences with h = 1e-4 for w_A, w_B,
    L (GPU FP64 losses), fA (reference continuous relaxation) and chi (zero)."""
    dims, shape = (96, 96, 96), (96, 96, 96)
    rng = np.random.default_rng(96)
    fields = {m: 0.1 * rng.standard_normal(shape) for m in (1, 2)}
    target = AD.smooth_target(shape, 0.35, amp=0.2, nmodes=5, seed=12345)

    def make(M, precision=None, L=8.0, NA=35.0, chi=0.2):
        A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
        cell = M.UnitCell(3, "cubic", L)
        s = M.FieldSystem(dims, cell, monomers=[A, B]) if precision is None else \
            M.FieldSystem(dims, cell, monomers=[A, B], precision=precision)
        s.add_species(M.Multiblock([A, B], [NA, 100.0 - NA], [1.0, 1.0], 200), 1.0)
        itx = M.FloryInteraction()
        itx.set_interaction(A, B, chi)
        s.add_interaction(itx)
        for m in (1, 2):
            s.fields[m] = fields[m].copy() if M is O else fields[m]
        return s

    o = make(O)
    o.density_update()
    _, rbar = AD.density_loss(o, 1, target)
    go = AD.density_pullback(o, rbar)
    s64, s32 = make(pf, "fp64"), make(pf, "fp32")
    s64.set_adjoint_checkpoints(15)  # q checkpointed every 15 contour steps
    s32.set_adjoint_checkpoints(15)
    g64 = s64.density_pullback(rbar)
    g32 = s32.density_pullback(rbar)
    del s64, s32
    for m in (1, 2):
        assert relmax(g64["w"][m], go["w"][m]) < 1e-9
        assert relmax(g32["w"][m], go["w"][m]) < 1e-3
    assert relmax(g64["cell"], go["cell"]) < 1e-9
    assert relmax(g32["cell"], go["cell"]) < 1e-3
    dfa64 = 100.0 * (g64["Nref_block"][0][0] - g64["Nref_block"][0][1])
    dfao = 100.0 * (go["Nref_block"][0][0] - go["Nref_block"][0][1])
    assert dfa64 == pytest.approx(dfao, rel=1e-9)

    h = 1e-4

    def gpu_loss(**kw):
        s = make(pf, "fp64", **kw)
        s.density_update()
        d = s.density[1] - target
        return float(np.sum(d * d))

    for m in (1, 2):
        for idx in [(3, 50, 17), (70, 8, 91)]:
            fp = {k: v.copy() for k, v in fields.items()}
            fm = {k: v.copy() for k, v in fields.items()}
            fp[m][idx] += h
            fm[m][idx] -= h
            sp_, sm_ = make(pf, "fp64"), make(pf, "fp64")
            sp_.fields[m], sm_.fields[m] = fp[m], fm[m]
            sp_.density_update()
            sm_.density_update()
            fd = (np.sum((sp_.density[1] - target) ** 2) - np.sum((sm_.density[1] - target) ** 2)) / (2 * h)
            assert g64["w"][m][idx] == pytest.approx(fd, rel=1e-5, abs=1e-9), (m, idx)
    fdL = (gpu_loss(L=8.0 + h) - gpu_loss(L=8.0 - h)) / (2 * h)
    assert g64["cell"][0] == pytest.approx(fdL, rel=1e-5)
    assert gpu_loss(chi=0.2 + h) == gpu_loss(chi=0.2 - h)  # dL/dchi = 0 at fixed fields

    def oracle_loss(NA):
        s = make(O, NA=NA)
        s.density_update()
        return AD.density_loss(s, 1, target)[0]

    fdf = (oracle_loss(35.0 + 100 * h) - oracle_loss(35.0 - 100 * h)) / (2 * h)
    assert dfa64 == pytest.approx(fdf, rel=1e-5)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("name,dims,crystal,params,blend", [CASES[2], CASES[4]], ids=[CASES[2][0], CASES[4][0]])
def test_checkpointed_pullback_equals_stored(name, dims, crystal, params, blend, prec):
    """Recomputing the propagators between checkpoints every 15 contour steps gives the same
    gradients as reading the stored histories (the recompute repeats the forward arithmetic)."""
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(33)
    mids = [1, 2, 3] if blend else [1, 2]
    fields = {m: 0.4 * rng.standard_normal(shape) for m in mids}
    rbar = {1: rng.standard_normal(shape), 2: rng.standard_normal(shape)}
    g = build(pf, dims, crystal, params, fields, blend, precision=prec)
    ref = g.density_pullback(rbar)
    g.set_adjoint_checkpoints(15)
    ck = g.density_pullback(rbar)
    tol = 1e-12 if prec == "fp64" else 1e-6
    for m in mids:
        assert relmax(ck["w"][m], ref["w"][m]) < tol, m
    assert relmax(ck["cell"], ref["cell"]) < tol


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-3)])
@pytest.mark.parametrize("name,dims,crystal,params,blend", CASES, ids=[c[0] for c in CASES])
def test_free_energy_pullback_matches_reference_gradient(name, dims, crystal, params, blend, prec, tol):
    """Gradient of free_energy (src/system/system.jl:402-433) at fixed fields: dF/dw, dF/dtheta,
    dF/dNref_b and dF/dchi against oracle/pf_adjoint.free_energy_pullback."""
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(23)
    mids = [1, 2, 3] if blend else [1, 2]
    fields = {m: 0.4 * rng.standard_normal(shape) for m in mids}
    o = build(O, dims, crystal, params, fields, blend)
    o.density_update()
    go = AD.free_energy_pullback(o)
    g = build(pf, dims, crystal, params, fields, blend, precision=prec)
    gg = g.free_energy_pullback()
    assert gg["fhelm"] == pytest.approx(o.free_energy(), rel=tol)
    for m in mids:
        assert relmax(gg["w"][m], go["w"][m]) < tol, (m, relmax(gg["w"][m], go["w"][m]))
    assert relmax(gg["cell"], go["cell"]) < tol
    for a, b in zip(gg["Nref_block"], go["Nref_block"]):
        if b:
            assert relmax(a, b) < tol
    assert gg["chi"][(1, 2)] == pytest.approx(go["chi"][(1, 2)], rel=tol)


def test_free_energy_pullback_96cubed():
    """Loss on fhelm for the differentiation workload (96^3, cubic L 8, AB diblock N100 fA0.35,
    Ns 200, chi 0.2): GPU FP64 against the FP64 CPU reference gradient (1e-9) and central
    differences (h = 1e-4) of GPU FP64 free energies for w_A, w_B, L and chi (which now has a
    nonzero derivative: chi enters fhelm through the Flory energy)."""
    dims, shape = (96, 96, 96), (96, 96, 96)
    rng = np.random.default_rng(97)
    fields = {m: 0.1 * rng.standard_normal(shape) for m in (1, 2)}

    def make(M, precision=None, L=8.0, chi=0.2):
        A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
        cell = M.UnitCell(3, "cubic", L)
        s = M.FieldSystem(dims, cell, monomers=[A, B]) if precision is None else \
            M.FieldSystem(dims, cell, monomers=[A, B], precision=precision)
        s.add_species(M.Multiblock([A, B], [35.0, 65.0], [1.0, 1.0], 200), 1.0)
        itx = M.FloryInteraction()
        itx.set_interaction(A, B, chi)
        s.add_interaction(itx)
        for m in (1, 2):
            s.fields[m] = fields[m].copy() if M is O else fields[m]
        return s

    o = make(O)
    o.density_update()
    go = AD.free_energy_pullback(o)
    s64 = make(pf, "fp64")
    s64.set_adjoint_checkpoints(15)
    g64 = s64.free_energy_pullback()
    del s64
    for m in (1, 2):
        assert relmax(g64["w"][m], go["w"][m]) < 1e-9
    assert relmax(g64["cell"], go["cell"]) < 1e-9
    assert g64["chi"][(1, 2)] == pytest.approx(go["chi"][(1, 2)], rel=1e-9)
    h = 1e-4

    def fh(fields_=None, **kw):
        s = make(pf, "fp64", **kw)
        if fields_ is not None:
            for m, w in fields_.items():
                s.fields[m] = w
        s.density_update()
        return s.free_energy()

    for m in (1, 2):
        idx = (5, 40, 77)
        fp = {k: v.copy() for k, v in fields.items()}
        fm = {k: v.copy() for k, v in fields.items()}
        fp[m][idx] += h
        fm[m][idx] -= h
        fd = (fh(fp) - fh(fm)) / (2 * h)
        assert g64["w"][m][idx] == pytest.approx(fd, rel=1e-4, abs=1e-11), (m, idx)
    assert g64["cell"][0] == pytest.approx((fh(L=8.0 + h) - fh(L=8.0 - h)) / (2 * h), rel=1e-5)
    assert g64["chi"][(1, 2)] == pytest.approx((fh(chi=0.2 + h) - fh(chi=0.2 - h)) / (2 * h), rel=1e-6)


def test_torch_autograd_free_energy_matches_pullback():
    torch = pytest.importorskip("torch")
    from polyfields import autodiff
    dims, shape = (32, 32, 1), (1, 32, 32)
    rng = np.random.default_rng(5)
    fields = {m: 0.3 * rng.standard_normal(shape) for m in (1, 2)}
    g = build(pf, dims, "hexagonal", [6.0], fields, precision="fp64")
    ws = {m: torch.tensor(fields[m], requires_grad=True) for m in (1, 2)}
    f = autodiff.free_energy(g, ws)
    f.backward()
    ref = build(pf, dims, "hexagonal", [6.0], fields, precision="fp64").free_energy_pullback()
    assert float(f) == pytest.approx(ref["fhelm"], rel=1e-12)
    for m in (1, 2):
        assert relmax(ws[m].grad.numpy(), ref["w"][m]) < 1e-12
