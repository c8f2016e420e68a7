"""Pins the FP64 oracle against the reference's own tests and published outputs.

Runs on the CPU only.  Every assertion cites the reference file the number comes from
(see tests/golden/reference_values.py).
"""
import math

import numpy as np
import pytest

import pf_oracle as O
import reference_values as RV


def _load_seed(golden_dir, name):
    d = np.load(f"{golden_dir}/seed_{name}.npz")
    fields = {int(k[1:]): d[k] for k in d.files if k.startswith("w")}
    return d, fields


# ----------------------------------------------------------------------------- unit tests
@pytest.mark.parametrize("args,vol", RV.CELL_VOLUMES)
def test_cell_volumes(args, vol):
    """test/test_cell.jl:3-36."""
    cell = O.UnitCell(*args)
    assert O.isapprox(cell.volume, vol)


def test_species_values():
    """test/test_species.jl:5-16."""
    amon = O.Monomer(1, vol=2.0)
    bmon = O.Monomer(2, vol=1.0)
    assert O.isapprox(O.Point(amon).Nref, RV.SPECIES["point_Nref"])
    assert O.isapprox(O.Homopolymer(bmon, 100, 1.0, 200).Nref, RV.SPECIES["homopolymer_Nref"])
    chain = O.Diblock(amon, bmon, 100, 0.25, 1.0, 1.0, 200)
    assert O.isapprox(chain.f_block[0], RV.SPECIES["diblock_f_block_1"])
    assert O.isapprox(chain.Nref_block[1], RV.SPECIES["diblock_Nref_block_2"])
    chain = O.Multiblock([amon, amon, bmon, amon, bmon, bmon], [10] * 6, [1.0] * 6, 60)
    assert O.isapprox(chain.monomer_fraction(1), RV.SPECIES["multiblock_fraction_1"])


def test_flory_pairs():
    """test/test_interactions.jl:1-6."""
    fh = O.FloryInteraction()
    fh.set_interaction(1, 2, 0.5)
    fh.set_interaction(2, 1, 0.5)
    assert len(fh.chis) == 1
    with pytest.raises(AssertionError):
        fh.set_interaction(1, 1, 0.5)


def test_diblock_trunc_error():
    """multiblock.jl:66-72: float trunc makes f=0.29 at N=100 fail."""
    a, b = O.Monomer(1), O.Monomer(2)
    with pytest.raises(ValueError):
        O.Diblock(a, b, 100, 0.29, 1.0, 1.0, 100)


def test_chain_grid_adjusts_ns():
    """multiblock.jl:56-59: N=100, f=0.35, Ns=100 is re-discretised to Ns=102."""
    a, b = O.Monomer(1), O.Monomer(2)
    ch = O.Diblock(a, b, 100, 0.35, 1.0, 1.0, 100)
    assert ch.Ns == 102
    ch = O.Diblock(a, b, 100, 0.35, 1.0, 1.0, 200)
    assert ch.Ns == 200 and ch.begin_block == [1, 71, 201]


# ----------------------------------------------------------------------------- FFT layout
def test_half_spectrum_layout_matches_dft():
    """rfft on x (fastest axis) with the (Nz, Ny, Kx) layout of src/utils.jl:9."""
    rng = np.random.default_rng(0)
    a = rng.standard_normal((3, 4, 6))
    k = O._rfftn(a, 1)
    assert k.shape == (3, 4, 4)
    z, y, x = np.meshgrid(np.arange(3), np.arange(4), np.arange(6), indexing="ij")
    for kz, ky, kx in [(0, 0, 0), (1, 2, 3), (2, 3, 1)]:
        ph = np.exp(-2j * np.pi * (kx * x / 6 + ky * y / 4 + kz * z / 3))
        assert abs(np.sum(a * ph) - k[kz, ky, kx]) < 1e-12


def test_lu_inverse_matches_numpy():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((7, 7))
    assert np.allclose(O.lu_inverse(A), np.linalg.inv(A), rtol=1e-12, atol=1e-12)
    with pytest.raises(np.linalg.LinAlgError):
        O.lu_inverse(np.zeros((3, 3)))


# ----------------------------------------------------------------------------- goldens
def _blend_system(golden_dir):
    d, fields = _load_seed(golden_dir, "abc_blend_1d")
    A, B, C = O.Monomer(1, 2.0), O.Monomer(2, 2.0), O.Monomer(3, 1.0)
    cell = O.UnitCell(int(d["dim"]), str(d["crystal"]), *d["cell_params"])
    sys = O.FieldSystem(tuple(d["grid"]), cell, monomers=[A, B, C])
    sys.add_species(O.Point(C), 0.4)
    sys.add_species(O.Homopolymer(A, 100, 1.0), 0.3)
    sys.add_species(O.Homopolymer(B, 100, 1.0), 0.3)
    itx = O.FloryInteraction()
    itx.set_interaction(A, B, 0.5)
    itx.set_interaction(A, C, 1.25)
    itx.set_interaction(B, C, 1.25)
    sys.add_interaction(itx)
    O.fieldinit(sys, fields)
    return sys


def test_blend_seed_reproduces_published_results(golden_dir):
    """examples/examples.ipynb cell 12: the saved converged blend gives back the printed
    SCFTResults.ferr and .fhelm (Point + two homopolymers + three chi pairs, quirk Q3)."""
    sys = _blend_system(golden_dir)
    assert sys.field_error() == pytest.approx(RV.BLEND_FINAL["ferr"], rel=1e-9)
    assert sys.free_energy() == pytest.approx(RV.BLEND_FINAL["fhelm"], rel=1e-12)


def test_cyl2d_seed_matches_published_fhelm(golden_dir):
    """examples/examples.ipynb cell 8: hexagonal cylinders (quirk Q1 fold).  The seed is
    64x64, the notebook ran 128x128, so agreement is to the spatial discretisation."""
    d, fields = _load_seed(golden_dir, "cyl2d")
    A, B = O.Monomer(1), O.Monomer(2)
    cell = O.UnitCell(2, "hexagonal", *d["cell_params"])
    assert d["cell_params"][0] == RV.CYL2D_FINAL_128["a"]
    sys = O.FieldSystem(tuple(d["grid"]), cell, monomers=[A, B])
    sys.add_species(O.Diblock(A, B, 100, 0.3, 1.0, 1.0, 100), 1.0)
    itx = O.FloryInteraction()
    itx.set_interaction(A, B, 0.3)
    sys.add_interaction(itx)
    O.fieldinit(sys, fields)
    assert sys.field_error() < 1.1e-5
    assert abs(sys.free_energy() - RV.CYL2D_FINAL_128["fhelm"]) < 1e-8


def test_lam1d_seed_matches_published_fhelm(golden_dir):
    """examples/examples.ipynb cell 4 (the notebook interpolated the 64-point seed to 128)."""
    d, fields = _load_seed(golden_dir, "lam1d")
    A, B = O.Monomer(1), O.Monomer(2)
    cell = O.UnitCell(1, "lamellar", *d["cell_params"])
    sys = O.FieldSystem(tuple(d["grid"]), cell, monomers=[A, B])
    sys.add_species(O.Diblock(A, B, 100, 0.5, 1.0, 1.0, 100), 1.0)
    itx = O.FloryInteraction()
    itx.set_interaction(A, B, 0.25)
    sys.add_interaction(itx)
    O.fieldinit(sys, fields)
    assert sys.field_error() < 1.1e-5
    assert abs(sys.free_energy() - RV.LAM1D_FINAL_128["fhelm"]) < 1e-7


def _lamellar(L, n=64, chi=0.2, Ns=100):
    A, B = O.Monomer(1), O.Monomer(2)
    sys = O.FieldSystem((n, 1, 1), O.UnitCell(1, "lamellar", L), monomers=[A, B])
    sys.add_species(O.Diblock(A, B, 100, 0.5, 1.0, 1.0, Ns), 1.0)
    itx = O.FloryInteraction()
    itx.set_interaction(A, B, chi)
    sys.add_interaction(itx)
    x = np.arange(n) / n
    w = np.broadcast_to(np.cos(2 * np.pi * x), sys.shape).copy()
    O.fieldinit(sys, {1: w, 2: -w})
    return sys


def test_readme_converged_lamellar():
    """README.md:62-79: at the published converged cell the converged fields give the
    published free energy (to the published ferr ~ 5e-6) and a stress of the size of the
    published serr."""
    sys = _lamellar(RV.README_LAMELLAR["L"])
    res = O.scft(sys, O.AndersonUpdater(nhist=10), opts=O.SCFTOptions(nsteps=300, ftol=1e-10))
    assert res.converged
    assert abs(res.fhelm - RV.README_LAMELLAR["fhelm"]) < 5e-8
    assert abs(sys.scfstress()[0]) < 5 * RV.README_LAMELLAR["serr"]


def test_readme_scft_with_domain_updater():
    """The README run itself (Anderson nhist 10 + DomainUpdater nskip 5 / nper 20, ftol =
    stol = 1e-4) from a seeded start converges to the published lamellar state."""
    A, B = O.Monomer(1), O.Monomer(2)
    cell = O.UnitCell(1, "lamellar", 10.0)
    sys = O.FieldSystem((64, 1, 1), cell, monomers=[A, B])
    sys.add_species(O.Diblock(A, B, 100, 0.5, 1.0, 1.0, 100), 1.0)
    itx = O.FloryInteraction()
    itx.set_interaction(A, B, 0.2)
    sys.add_interaction(itx)
    rng = np.random.Generator(np.random.PCG64(12345))
    O.fieldinit(sys, {1: 0.1 * rng.standard_normal(sys.shape), 2: 0.1 * rng.standard_normal(sys.shape)})
    res = O.scft(sys, O.AndersonUpdater(nhist=10), domain=O.DomainUpdater(nskip=5, nper=20),
                 opts=O.SCFTOptions(nsteps=1500, ftol=1e-4, stol=1e-4))
    assert res.converged and res.ferr < 1e-4 and res.serr < 1e-4
    assert abs(cell.params[0] - RV.README_LAMELLAR["L"]) < 0.2
    assert abs(res.fhelm - RV.README_LAMELLAR["fhelm"]) < 2e-4


# ----------------------------------------------------------------------------- invariants
def test_uniform_field_partition_function():
    """With uniform fields q_s = exp(-sum vol*w*ds) exactly (mde.jl:50), so
    Q = exp(-sum_blk vol*w_blk*ds_blk*nsteps_blk)."""
    A, B = O.Monomer(1), O.Monomer(2)
    sys = O.FieldSystem((16, 1, 1), O.UnitCell(1, "lamellar", 5.0), monomers=[A, B])
    ch = O.Diblock(A, B, 100, 0.3, 1.0, 1.0, 100)
    sys.add_species(ch, 1.0)
    sys.fields[1][...] = 0.7
    sys.fields[2][...] = -0.2
    sys.density_update()
    expect = 0.0
    for iblk in range(ch.nblocks):
        nst = ch.begin_block[iblk + 1] - ch.begin_block[iblk]
        expect += (0.7 if iblk == 0 else -0.2) * ch.ds_block[iblk] * nst
    assert ch.Q == pytest.approx(math.exp(-expect), rel=1e-13)


def test_q_from_any_contour_point():
    """Q = mean(q_s * qc_s) for every s (a property of the exact propagators that the
    operator-split scheme keeps to rounding)."""
    sys = _lamellar(12.0, n=32)
    ch = sys.species[0]
    sys.density_update()
    for s in (0, 17, 50, 100):
        assert float(np.mean(ch.q[s] * ch.qc[s])) == pytest.approx(ch.Q, rel=1e-12)


def test_stress_is_free_energy_derivative():
    """At converged fields the stress of src/system/system.jl:384-395 is d f / dL of the
    free energy with the translational term phi*(mu - 1)/Nref, mu = log(phi/Q).  The
    reference's free_energy uses mu = phi there (quirk Q3), so the test adds the
    difference back before differentiating."""
    def f_true(sys):
        ch = sys.species[0]
        phi = sys.phi_species[0]
        return (sys.free_energy() - phi * (phi - 1.0) / ch.Nref
                + phi * (math.log(phi / ch.Q) - 1.0) / ch.Nref)

    # the Simpson-quadrature stress and the derivative of the operator-split Q differ at
    # O(ds^2): 1% at ds = 1, 0.06% at ds = 0.25
    h = 1e-3
    for Ns, rel in ((100, 2e-2), (400, 1.5e-3)):
        f = []
        for L in (15.0 - h, 15.0 + h):
            sys = _lamellar(L, Ns=Ns)
            O.scft(sys, O.AndersonUpdater(nhist=10), opts=O.SCFTOptions(nsteps=300, ftol=1e-11))
            f.append(f_true(sys))
        sys = _lamellar(15.0, Ns=Ns)
        O.scft(sys, O.AndersonUpdater(nhist=10), opts=O.SCFTOptions(nsteps=300, ftol=1e-11))
        fd = (f[1] - f[0]) / (2 * h)
        assert sys.scfstress()[0] == pytest.approx(fd, rel=rel)


def test_rqm4_more_accurate_than_rk2():
    """The Richardson scheme of mde.jl:83-104 converges faster in ds than RK2."""
    def Q(method, Ns):
        A = O.Monomer(1)
        sys = O.FieldSystem((32, 1, 1), O.UnitCell(1, "lamellar", 8.0), monomers=[A], mde=method)
        ch = O.Homopolymer(A, 100, 1.0, Ns)
        sys.add_species(ch, 1.0)
        x = np.arange(32) / 32
        sys.fields[1][...] = 0.3 * np.cos(2 * np.pi * x)
        sys.density_update()
        return ch.Q
    exact = Q("RQM4", 1600)
    assert abs(Q("RQM4", 50) - exact) < abs(Q("RK2", 50) - exact) / 10


# ----------------------------------------------------------------------------- quirk Q1 option
@pytest.mark.parametrize("dims,crystal,params", [((16, 16, 1), "hexagonal", (9.0,)),
                                                 ((12, 8, 1), "oblique", (7.0, 5.0, 1.2)),
                                                 ((8, 6, 6), "triclinic", (5.0, 4.0, 3.0, 1.4, 1.7, 1.3))])
def test_signed_frequency_option(dims, crystal, params):
    """Quirk Q1 (cell.jl:276-277, 306-307): the reference folds the y and z frequencies to |j|,
    which changes |k|^2 in non-orthogonal cells.  The signed option uses j - N above N/2;
    ksq then equals |G j|^2 over signed integer frequencies, differs from the folded ksq, and
    dksq stays the parameter derivative of ksq (central differences)."""
    def cell(p, signed):
        c = O.UnitCell(sum(1 for d in dims if d > 1), crystal, *p)
        c.setup(dims)
        c.set_signed_k(signed)
        return c
    c = cell(params, True)
    kx, ny, nz = O.ksize(dims)
    jx = np.arange(kx)[None, None, :]
    jy = np.array([i if i <= ny / 2 else i - ny for i in range(ny)])[None, :, None]
    jz = np.array([i if i <= nz / 2 else i - nz for i in range(nz)])[:, None, None]
    k = [c.G[r, 0] * jx + c.G[r, 1] * jy + c.G[r, 2] * jz for r in range(3)]
    assert np.allclose(c.ksq, k[0] ** 2 + k[1] ** 2 + k[2] ** 2, rtol=1e-13, atol=1e-12)
    assert not np.allclose(c.ksq, cell(params, False).ksq)
    h = 1e-6
    for p in range(len(params)):
        up, dn = list(params), list(params)
        up[p] += h
        dn[p] -= h
        fd = (cell(up, True).ksq - cell(dn, True).ksq) / (2 * h)
        assert np.allclose(c.dksq[p], fd, rtol=1e-6, atol=1e-6 * np.max(np.abs(fd))), p


def test_signed_frequency_option_changes_nothing_in_orthogonal_cells():
    for dims, crystal, params in (((32, 1, 1), "lamellar", (10.0,)), ((16, 8, 1), "rectangular", (9.0, 5.0)),
                                  ((8, 8, 8), "cubic", (6.0,))):
        a = O.UnitCell(sum(1 for d in dims if d > 1), crystal, *params)
        a.setup(dims)
        b = O.UnitCell(sum(1 for d in dims if d > 1), crystal, *params)
        b.setup(dims)
        b.set_signed_k(True)
        assert np.array_equal(a.ksq, b.ksq)
        for x, y in zip(a.dksq, b.dksq):
            assert np.array_equal(x, y)
