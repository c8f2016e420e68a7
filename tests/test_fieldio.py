"""Field IO of src/fileio.jl and src/utils.jl: interpolate_grid, loadfields, fieldinit from a path
or from densities, and the nsave checkpoints of scft! (simulate.jl:124-128).

interpolate_grid follows the reference's Interpolations.jl call, BSpline(Cubic(Line(OnGrid()))),
whose interpolant on the grid points is the natural cubic spline (zero second derivative at the
ends): checked against SciPy's natural CubicSpline, axis by axis (the tensor-product spline
factorises)."""
import json

import numpy as np
import pytest

pf = pytest.importorskip("polyfields")
from polyfields import api  # noqa: E402


def _scipy_resample(g, out_shape):
    interp = pytest.importorskip("scipy.interpolate")
    a = g
    for axis, (nin, nout) in enumerate(zip(g.shape, out_shape)):
        if nin == nout:
            continue
        a = interp.CubicSpline(np.arange(nin), a, axis=axis, bc_type="natural")(np.linspace(0, nin - 1, nout))
    return a


@pytest.mark.parametrize("shape,dims", [((1, 1, 7), (13, 1, 1)), ((1, 1, 64), (32, 1, 1)),
                                        ((1, 24, 32), (48, 16, 1)), ((6, 8, 10), (16, 12, 9))])
def test_interpolate_grid_is_the_natural_cubic_spline(shape, dims):
    g = np.random.default_rng(3).standard_normal(shape)
    out = pf.interpolate_grid(g, dims)
    assert out.shape == (dims[2], dims[1], dims[0])
    assert np.max(np.abs(out - _scipy_resample(g, out.shape))) < 1e-13


def test_interpolate_grid_endpoints_and_linear_data():
    """Output points run from the first to the last input point; linear data is reproduced."""
    x = np.linspace(-1.0, 2.0, 9)
    out = pf.interpolate_grid(x.reshape(1, 1, 9), (17, 1, 1)).ravel()
    assert np.allclose(out, np.linspace(-1.0, 2.0, 17), rtol=0, atol=1e-14)


def test_interpolate_grid_copies_and_slices_across_dimensions():
    g = np.random.default_rng(4).standard_normal((1, 8, 8))
    with pytest.warns(UserWarning, match="different dimensions"):
        up = pf.interpolate_grid(g, (8, 8, 4))
    assert up.shape == (4, 8, 8) and all(np.array_equal(up[k], g[0]) for k in range(4))
    h = np.random.default_rng(5).standard_normal((4, 8, 8))
    with pytest.warns(UserWarning):
        down = pf.interpolate_grid(h, (8, 8, 1))
    assert np.array_equal(down[0], h[0])


def test_loadfields_reads_the_reference_layout(tmp_path):
    f = np.arange(2 * 3 * 4, dtype=float).reshape(2, 3, 4)  # (Nz, Ny, Nx)
    doc = {"dim": 3, "grid": [4, 3, 2], "mids": [1], "date": "", "crystal": "orthorhombic",
           "cell_params": [4.0, 3.0, 2.0], "field_type": "omega", "fields": {"1": f.tolist()}}
    p = tmp_path / "seed.json"
    p.write_text(json.dumps(doc))
    d = pf.loadfields(str(p))
    assert d["grid"] == (4, 3, 2) and d["mids"] == [1] and d["crystal"] == "orthorhombic"
    assert np.array_equal(d["fields"][1], f)


def test_potentials_from_densities_restate_flory_and_edwards():
    """The host restatement used by fieldinit(field_type="rho") on a stand-in system."""
    class _Sys:
        shape = (1, 1, 4)
        monomers = {1: pf.Monomer(1, 1.0), 2: pf.Monomer(2, 2.0)}
        interactions = []
    s = _Sys()
    fl = pf.FloryInteraction()
    fl.set_interaction(1, 2, 0.3)
    ed = pf.EdwardsInteraction()
    ed.set_interaction(2, 5.0)
    s.interactions = [fl, ed]
    rho = {1: np.full(s.shape, 0.4), 2: np.full(s.shape, 0.6)}
    pots = api._potentials_from(s, rho)
    assert np.allclose(pots[1], 0.3 * 0.6 / 2.0)
    assert np.allclose(pots[2], 0.3 * 0.4 / 1.0 + 5.0 * 0.6 / 2.0)


def test_monomer_fraction_free_function_matches_species():
    A, B = pf.Monomer(1), pf.Monomer(2)
    chain = pf.Diblock(A, B, 100, 0.3, 1.0, 1.0, 100)
    assert pf.monomer_fraction(chain, 1) == pytest.approx(0.3)
    assert pf.monomer_fraction(chain, 2) == pytest.approx(0.7)
    assert pf.monomer_fraction(chain, 3) == 0.0
