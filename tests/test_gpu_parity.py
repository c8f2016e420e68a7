"""GPU engine vs the FP64 oracle on identical seeded inputs (through the C ABI).

Tolerances: FP64 propagators match the oracle to 1e-10 relative (the bar for the FP64 path);
FP32 propagators to 5e-5 relative on Q and densities (float32 rounding over 100-200 contour
steps), with all reductions in float64.
"""
import numpy as np
import pytest

import pf_oracle as O
import reference_values as RV
import systems as SY

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_RTOL = 5e-5


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


CASES = [
    ("lam1d_64", dict(dims=(64, 1, 1), crystal="lamellar", params=(10.0,))),
    ("lam1d_32_f03", dict(dims=(32, 1, 1), crystal="lamellar", params=(7.0,), f=0.3, chi=0.25)),
    ("hex2d_32", dict(dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), f=0.3, chi=0.3)),
    ("rect2d_64x32", dict(dims=(64, 32, 1), crystal="rectangular", params=(12.0, 7.0))),
    ("cubic3d_16", dict(dims=(16, 16, 16), crystal="cubic", params=(6.0,), f=0.3, amp=0.15)),
    ("cubic3d_32", dict(dims=(32, 32, 32), crystal="cubic", params=(7.0,), f=0.3, Ns=60, amp=0.15)),
]


@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_propagate_matches_oracle(name, kw):
    """PseudoSpectralSolver update! + propagate! (mde.jl:43-81), several contour steps."""
    dims = kw["dims"]
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(7)
    w = 0.3 * rng.standard_normal(shape)
    q0 = 1.0 + 0.1 * rng.standard_normal(shape)
    nd = sum(1 for d in dims if d > 1)
    ocell = O.UnitCell(nd, kw["crystal"], *kw["params"])
    ocell.setup(dims)
    solver = O.PseudoSpectralSolver(dims)
    solver.update(w, ocell.ksq, 1.3, 1.1, 0.5)
    q = q0.copy()
    out = np.empty(shape)
    for _ in range(5):
        solver.propagate(q, out)
        q = out.copy()
    for prec, tol in (("fp64", FP64_RTOL), ("fp32", FP32_RTOL)):
        sys = pf.FieldSystem(dims, pf.UnitCell(nd, kw["crystal"], *kw["params"]), precision=prec)
        got = np.empty(shape)
        L = pf.load_library()
        st = L.pf_propagate(sys._h, w.ctypes.data_as(pf._lib._dptr), 1.3, 1.1, 0.5,
                            q0.ctypes.data_as(pf._lib._dptr), got.ctypes.data_as(pf._lib._dptr), 5)
        pf._lib.check(st, sys._h)
        assert rel(got, q) < tol, (prec, rel(got, q))


@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_density_residuals_energy_fp64(name, kw):
    """density!, residuals!, free_energy, field_error and scfstress after fieldinit!."""
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=FP64_RTOL)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < FP64_RTOL
        assert rel(g.fields[mid], o.fields[mid]) < FP64_RTOL
        assert rel(g.residuals[mid], o.residuals[mid]) < 1e-9
        assert rel(g.potentials[mid], o.potentials[mid]) < FP64_RTOL
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=FP64_RTOL)
    assert g.field_error() == pytest.approx(o.field_error(), rel=1e-9)
    assert g.free_energy_bulk() == pytest.approx(o.free_energy_bulk(), rel=1e-13)
    so, sg = o.scfstress(), g.scfstress()
    assert np.allclose(sg, so, rtol=1e-9, atol=1e-14 * max(1.0, np.max(np.abs(so))))


@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_propagators_per_step_fp64(name, kw):
    """Every stored q_s and qc_s of the forward and backward passes (multiblock.jl:136-171)."""
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    ch_o, ch_g = o.species[0], g.species[0]
    for s in sorted({0, 1, ch_o.Ns // 3, ch_o.Ns // 2, ch_o.Ns - 1, ch_o.Ns}):
        assert rel(ch_g.propagator(s), ch_o.q[s]) < FP64_RTOL
        assert rel(ch_g.propagator(s, conjugate=True), ch_o.qc[s]) < FP64_RTOL


@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_density_fp32(name, kw):
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp32", **kw)
    assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=FP32_RTOL)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < FP32_RTOL
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=1e-4)


def test_blend_seed_golden_gpu():
    """examples/examples.ipynb cell 12 published ferr/fhelm, on the GPU (Point + homopolymers)."""
    g = SY.blend_seed_system(pf, precision="fp64")
    o = SY.blend_seed_system(O)
    assert g.field_error() == pytest.approx(RV.BLEND_FINAL["ferr"], rel=1e-9)
    assert g.free_energy() == pytest.approx(RV.BLEND_FINAL["fhelm"], rel=1e-12)
    for isp in range(3):
        assert g.species[isp].Q == pytest.approx(o.species[isp].Q, rel=FP64_RTOL)
    for mid in (1, 2, 3):
        assert rel(g.density[mid], o.density[mid]) < FP64_RTOL


def test_cyl2d_seed_gpu():
    """examples/examples.ipynb cell 8 (hexagonal, quirk Q1 fold) on the GPU."""
    g = SY.cyl2d_seed_system(pf, precision="fp64")
    o = SY.cyl2d_seed_system(O)
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=FP64_RTOL)
    assert abs(g.free_energy() - RV.CYL2D_FINAL_128["fhelm"]) < 1e-8
    assert np.allclose(g.scfstress(), o.scfstress(), rtol=1e-9, atol=1e-15)


def test_blend3d_density_fp64():
    """Two species (diblock + homopolymer, Ns=200) on a 3D grid: both chains in one launch.
    The stress carries quirk Q2 (multiblock.jl:279-282: Re*Re products only, and every
    half-spectrum entry after the k = 0 one doubled, the kx = 0 and Nyquist planes included),
    as the oracle does."""
    o = SY.blend3d_system(O, n=16)
    g = SY.blend3d_system(pf, n=16, precision="fp64")
    for isp in range(2):
        assert g.species[isp].Q == pytest.approx(o.species[isp].Q, rel=FP64_RTOL)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < FP64_RTOL
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=FP64_RTOL)
    assert np.allclose(g.scfstress(), o.scfstress(), rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("name,kw", CASES[:5], ids=[c[0] for c in CASES[:5]])
def test_anderson_steps_fp64(name, kw):
    """10 AndersonUpdater steps (anderson.jl:98-228) including the Euler warm-up, the history
    fill and the shift (nhist = 4)."""
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    uo = O.AndersonUpdater(nhist=4)
    uo.setup(o)
    ug = pf.AndersonUpdater(nhist=4)
    ug.setup(g)
    for _ in range(10):
        uo.step()
        ug.step()
    for mid in (1, 2):
        assert rel(g.fields[mid], o.fields[mid]) < 1e-8
        assert rel(g.residuals[mid], o.residuals[mid]) < 1e-7
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=1e-9)


def test_scft_domain_lamellar_fp64():
    """scft! with Anderson + DomainUpdater on the README lamellar case (README.md:62-79).

    Quirk Q4: DomainUpdater.step! never stops early, so both sides run nper Newton
    iterations per update (domain.jl:59-89).
    The DomainUpdater's finite-difference Jacobian (dx = 1e-8, domain.jl:101) multiplies the
    rounding error of the stress by 1e8, so two correct FP64 implementations that sum in a
    different order follow cell trajectories that agree to ~1e-7 relative, not to 1e-10."""
    kw = dict(dims=(64, 1, 1), crystal="lamellar", params=(10.0,), scale=0.1, amp=0.0)
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    opts_o = O.SCFTOptions(nsteps=400, ftol=1e-4, stol=1e-4)
    opts_g = pf.SCFTOptions(nsteps=400, ftol=1e-4, stol=1e-4)
    ro = O.scft(o, O.AndersonUpdater(nhist=10), domain=O.DomainUpdater(nskip=5, nper=20), opts=opts_o)
    rg = pf.scft(g, pf.AndersonUpdater(nhist=10), domain=pf.DomainUpdater(nskip=5, nper=20), opts=opts_g)
    assert rg.converged and ro.converged
    assert rg.nsteps == ro.nsteps
    assert rg.fhelm == pytest.approx(ro.fhelm, rel=1e-6)
    assert g.cell.params[0] == pytest.approx(o.cell.params[0], rel=1e-6)
    assert abs(rg.fhelm - RV.README_LAMELLAR["fhelm"]) < 2e-4


def test_scft_readme_converged_cell_fp64():
    """At the README's converged cell the GPU converges to the published free energy."""
    kw = dict(dims=(64, 1, 1), crystal="lamellar", params=(RV.README_LAMELLAR["L"],), scale=0.0, amp=1.0)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    r = pf.scft(g, pf.AndersonUpdater(nhist=10), opts=pf.SCFTOptions(nsteps=300, ftol=1e-10))
    assert r.converged
    assert abs(r.fhelm - RV.README_LAMELLAR["fhelm"]) < 5e-8


def test_mixed_precision_reaches_fp64_answer():
    """FP32 iterations then FP64 polish reach the FP64 fixed point (|dfhelm| <= 1e-8)."""
    kw = dict(dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), f=0.3, chi=0.3)
    g64 = SY.diblock_system(pf, precision="fp64", **kw)
    r64 = pf.scft(g64, pf.AndersonUpdater(nhist=10), opts=pf.SCFTOptions(nsteps=2000, ftol=1e-8))
    gm = SY.diblock_system(pf, precision="fp32", **kw)
    rm = pf.scft(gm, pf.AndersonUpdater(nhist=10),
                 opts=pf.SCFTOptions(nsteps=2000, ftol=1e-8, mixed_switch_ferr=1e-5))
    assert r64.converged and rm.converged
    assert rm.switch_step >= 0
    assert abs(rm.fhelm - r64.fhelm) <= 1e-8


def test_nan_field_raises():
    """scft! stops with the reference's error on a diverging (NaN) field (simulate.jl:109-111)."""
    kw = dict(dims=(32, 1, 1), crystal="lamellar", params=(10.0,))
    g = SY.diblock_system(pf, precision="fp64", **kw)
    w = g.fields[1]
    w[0, 0, 3] = np.nan
    g.fields[1] = w
    with pytest.raises(pf.PolyFieldsError, match="Diverging field updater"):
        pf.scft(g, pf.AndersonUpdater(nhist=5), opts=pf.SCFTOptions(nsteps=5, ftol=1e-12))


def test_singular_gram_raises():
    """Identical residual history makes Umn singular: the reference's LU error (anderson.jl:184-189).
    Fields that are already exact fixed points give zero residual differences."""
    A = pf.Monomer(1)
    g = pf.FieldSystem((16, 1, 1), pf.UnitCell(1, "lamellar", 5.0), monomers=[A])
    g.add_species(pf.Homopolymer(A, 10, 1.0, 10), 1.0)
    pf.fieldinit(g, {1: np.full(g.shape, 1e-3)})
    u = pf.AndersonUpdater(nhist=3)
    u.setup(g)
    u.step()
    with pytest.raises(pf.PolyFieldsError, match="Error inverting Umn"):
        u.step()


def test_fp32_rescaled_strong_fields():
    """Strong double-gyroid fields make Q ~ 1e40+, beyond float32's range: the FP32 chains
    are rescaled per contour step and the factors are carried in FP64 (Q, density, stress)."""
    o = SY.blend3d_system(O, n=16)
    g = SY.blend3d_system(pf, n=16, precision="fp32")
    assert o.species[0].Q > 1e30
    # 400 float32 contour steps through fields of this strength: 1e-4 on Q
    for isp in range(2):
        assert g.species[isp].Q == pytest.approx(o.species[isp].Q, rel=2 * FP32_RTOL)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < 2 * FP32_RTOL
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=1e-4)
    assert np.allclose(g.scfstress(), o.scfstress(), rtol=2e-3, atol=1e-9)


def test_fp32_propagator_accessor_unscaled():
    """chain.q[s] / qc[s] read back from rescaled FP32 histories equal the true propagators."""
    kw = dict(dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), f=0.3, chi=0.3)
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp32", **kw)
    ch_o, ch_g = o.species[0], g.species[0]
    for s in (0, 7, 50, ch_o.Ns):
        assert rel(ch_g.propagator(s), ch_o.q[s]) < FP32_RTOL
        assert rel(ch_g.propagator(s, conjugate=True), ch_o.qc[s]) < FP32_RTOL


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_RTOL), ("fp32", FP32_RTOL)])
def test_density_graph_replay_follows_fields_and_cell(prec, tol):
    """From the third density solve on, the engine replays one captured CUDA graph per
    precision.  New fields (read by the graph from the same buffers) and new cells (bond
    operators regenerated outside the graph) must still give the oracle's densities."""
    kw = dict(dims=(16, 16, 16), crystal="cubic", params=(6.0,), f=0.3, amp=0.15)
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision=prec, **kw)
    shape = o.shape
    for k in range(6):
        if k in (3, 5):
            o.add_cell(O.UnitCell(3, "cubic", 6.0 + 0.1 * k))
            g.add_cell(pf.UnitCell(3, "cubic", 6.0 + 0.1 * k))
        fields = SY.seeded_fields(shape, [1, 2], seed=200 + k, scale=0.2)
        O.fieldinit(o, fields)
        pf.fieldinit(g, fields)
        o.density_update()
        g.density_update()
        assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=tol), k
        for mid in (1, 2):
            assert rel(g.density[mid], o.density[mid]) < tol, (k, mid)


UPDATERS = [("euler_PEC", "Euler", dict(method="PEC", lam=0.05)), ("euler_PECE", "Euler", dict(method="PECE", lam=0.05)),
            ("mom", "Momentum", dict(method="MOM", lam=0.05)), ("rms", "Momentum", dict(method="RMS", lam=0.005)),
            ("adam", "Momentum", dict(method="ADAM", lam=0.005)), ("nag", "Momentum", dict(method="NAG", lam=0.05))]


@pytest.mark.parametrize("case", [CASES[2], CASES[4]], ids=[CASES[2][0], CASES[4][0]])
@pytest.mark.parametrize("uname,kind,ukw", UPDATERS, ids=[u[0] for u in UPDATERS])
def test_euler_momentum_steps_fp64(uname, kind, ukw, case):
    """12 steps of EulerUpdater (euler.jl:37-65, predictor on the updated field as the
    reference does) and MomentumUpdater (momentum.jl:63-165) against the oracle."""
    name, kw = case
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    uo = O.EulerUpdater(**ukw) if kind == "Euler" else O.MomentumUpdater(**ukw)
    ug = pf.EulerUpdater(**ukw) if kind == "Euler" else pf.MomentumUpdater(**ukw)
    uo.setup(o)
    ug.setup(g)
    for _ in range(12):
        uo.step()
        ug.step()
    for mid in (1, 2):
        assert rel(g.fields[mid], o.fields[mid]) < 1e-9, mid


def test_scft_with_euler_updater_fp64():
    """scft! drives any field updater (simulate.jl:60-148): EulerUpdater(:PECE) on the README
    lamellar system reaches the oracle's state step for step."""
    kw = dict(dims=(64, 1, 1), crystal="lamellar", params=(10.0,))
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    ro = O.scft(o, O.EulerUpdater(method="PECE", lam=0.1), opts=O.SCFTOptions(nsteps=60, ftol=1e-12))
    rg = pf.scft(g, pf.EulerUpdater(method="PECE", lam=0.1), opts=pf.SCFTOptions(nsteps=60, ftol=1e-12))
    assert rg.nsteps == ro.nsteps
    assert rg.fhelm == pytest.approx(ro.fhelm, rel=1e-10)
    for mid in (1, 2):
        assert rel(g.fields[mid], o.fields[mid]) < 1e-9


@pytest.mark.parametrize("name,kw", [CASES[0], CASES[2], CASES[4]], ids=[CASES[0][0], CASES[2][0], CASES[4][0]])
def test_rqm4_density_fp64(name, kw):
    """FieldSystem(...; mde = :RQM4): Richardson extrapolation (4 q2 - q1) / 3 of one full and two
    half RK2 steps per contour step (mde.jl:83-104), float64 chains: Q, densities, free energy
    and stress against the oracle's RQM4 solver."""
    def build(M, **extra):
        A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
        dims = kw["dims"]
        nd = sum(1 for d in dims if d > 1)
        s = M.FieldSystem(dims, M.UnitCell(nd, kw["crystal"], *kw["params"]), monomers=[A, B], mde="RQM4", **extra)
        s.add_species(M.Diblock(A, B, 100, kw.get("f", 0.5), 1.0, 1.0, 100), 1.0)
        itx = M.FloryInteraction()
        itx.set_interaction(A, B, kw.get("chi", 0.2))
        s.add_interaction(itx)
        shape = (dims[2], dims[1], dims[0])
        M.fieldinit(s, SY.seeded_fields(shape, [1, 2], 31, 0.3))
        return s
    o = build(O)
    g = build(pf, precision="fp64")
    assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=FP64_RTOL)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < FP64_RTOL
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=FP64_RTOL)
    assert np.allclose(g.scfstress(), o.scfstress(), rtol=1e-9, atol=1e-14)


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_RTOL), ("fp32", FP32_RTOL)])
def test_edwards_interaction(prec, tol):
    """EdwardsInteraction (edwards.jl:34-87) beside a FloryInteraction: potentials, residuals,
    free energy (the (u/2) sum (rho/v)^2 term) and bulk free energy against the oracle."""
    def build(M, **extra):
        A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.3)
        s = M.FieldSystem((32, 32, 1), M.UnitCell(2, "hexagonal", 8.0), monomers=[A, B], **extra)
        s.add_species(M.Diblock(A, B, 100, 0.5, 1.0, 1.0, 100), 1.0)
        f = M.FloryInteraction()
        f.set_interaction(A, B, 0.25)
        s.add_interaction(f)
        e = M.EdwardsInteraction()
        e.set_interaction(A, 0.6)
        e.set_interaction(B, 0.3)
        s.add_interaction(e)
        M.fieldinit(s, SY.seeded_fields((1, 32, 32), [1, 2], 41, 0.3))
        return s
    o = build(O)
    g = build(pf, precision=prec)
    for mid in (1, 2):
        assert rel(g.potentials[mid], o.potentials[mid]) < tol
        assert rel(g.residuals[mid], o.residuals[mid]) < 10 * tol
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=tol)
    assert g.free_energy_bulk() == pytest.approx(o.free_energy_bulk(), rel=1e-13)


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_RTOL), ("fp32", 2 * FP32_RTOL)])
def test_grand_ensemble(prec, tol):
    """Grand ensemble (system.jl:148-157, 248-259, 332-339): add_species! values are chemical
    potentials, phi = Q exp(mu) after each solve, no mean subtraction; a diblock, a homopolymer
    and a point species, 2D hexagonal cell."""
    def build(M, **extra):
        A, B, C = M.Monomer(1, 1.0), M.Monomer(2, 1.0), M.Monomer(3, 1.0)
        ens = O.GRAND if M is O else pf.Grand
        s = M.FieldSystem((32, 32, 1), M.UnitCell(2, "hexagonal", 8.0), monomers=[A, B, C], ensemble=ens, **extra)
        s.add_species(M.Diblock(A, B, 100, 0.4, 1.0, 1.0, 100), -5.8)
        s.add_species(M.Homopolymer(A, 50, 1.0, 100), -1.3)
        s.add_species(M.Point(C), -0.5)
        f = M.FloryInteraction()
        f.set_interaction(A, B, 0.2)
        f.set_interaction(B, C, 0.1)
        s.add_interaction(f)
        M.fieldinit(s, SY.seeded_fields((1, 32, 32), [1, 2, 3], 43, 0.3))
        return s
    o = build(O)
    g = build(pf, precision=prec)
    for mid in (1, 2, 3):
        assert rel(g.density[mid], o.density[mid]) < tol, mid
        assert rel(g.residuals[mid], o.residuals[mid]) < 10 * tol, mid
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=tol)
    assert np.allclose(g.scfstress(), o.scfstress(), rtol=1e-9 if prec == "fp64" else 2e-3, atol=1e-12)


def test_pencil_schedule_is_autotuned_on_first_solve():
    """The first density solve on a 3D grid tunes the pencil pass's schedule (stages x tiles
    per CTA) by timing real contour steps; later solves use it and still match the oracle."""
    kw = dict(dims=(32, 32, 32), crystal="cubic", params=(7.0,), f=0.3, Ns=60, amp=0.15)
    g = SY.diblock_system(pf, precision="fp32", **kw)
    stages, rounds, tuned = g.pencil_schedule()
    assert tuned and stages in (2, 3) and rounds in (1, 2, 4)
    o = SY.diblock_system(O, **kw)
    o.density_update()
    for _ in range(3):  # replayed graphs use the tuned schedule
        g.density_update()
    assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=FP32_RTOL)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < FP32_RTOL


def test_anderson_rejects_the_grand_ensemble():
    """AndersonUpdater setup! (anderson.jl:61-63) refuses a Grand-ensemble system with the
    reference's message, as the oracle does."""
    def build(M):
        A, B = M.Monomer(1, 1.0), M.Monomer(2, 1.0)
        ens = O.GRAND if M is O else pf.Grand
        s = M.FieldSystem((32, 1, 1), M.UnitCell(1, "lamellar", 8.0), monomers=[A, B], ensemble=ens)
        s.add_species(M.Diblock(A, B, 100, 0.5, 1.0, 1.0, 100), -1.0)
        f = M.FloryInteraction()
        f.set_interaction(A, B, 0.2)
        s.add_interaction(f)
        M.fieldinit(s, SY.seeded_fields((1, 1, 32), [1, 2], 7, 0.3))
        return s
    msg = "Anderson mixing can only be used for systems in the canonical ensemble."
    with pytest.raises(ValueError, match=msg):
        O.scft(build(O), O.AndersonUpdater(nhist=5), opts=O.SCFTOptions(nsteps=3))
    with pytest.raises(pf.PolyFieldsError, match=msg):
        pf.scft(build(pf), pf.AndersonUpdater(nhist=5), opts=pf.SCFTOptions(nsteps=3))
