"""fieldinit! from a seed file (with cell and interpolation), from densities, and the nsave
checkpoints of scft! (src/fileio.jl:25-97, src/simulate.jl:124-128) on the GPU engine."""
import json

import numpy as np
import pytest

import pf_oracle as O
import systems as SY

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _seed(path, grid, crystal, params, fields):
    doc = {"dim": sum(1 for n in grid if n > 1), "grid": list(grid), "mids": sorted(fields), "date": "",
           "crystal": crystal, "cell_params": list(params), "field_type": "omega",
           "fields": {str(m): f.tolist() for m, f in fields.items()}}
    path.write_text(json.dumps(doc))


def test_fieldinit_from_path_loads_cell_and_interpolates(tmp_path):
    g = SY.diblock_system(pf, dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), precision="fp64")
    rng = np.random.default_rng(11)
    seed = {1: rng.standard_normal((1, 24, 24)), 2: rng.standard_normal((1, 24, 24))}
    p = tmp_path / "seed.json"
    _seed(p, (24, 24, 1), "hexagonal", (8.5,), seed)
    pf.fieldinit(g, str(p))
    assert g.cell.params[0] == pytest.approx(8.5, rel=1e-15)
    for mid in (1, 2):
        want = pf.interpolate_grid(seed[mid], g.dims)
        assert rel(g.fields[mid], want - want.mean()) < 1e-13
    with pytest.raises(ValueError):
        pf.fieldinit(g, str(p), interpolate=False)


def test_fieldinit_from_densities_matches_oracle():
    """field_type = rho: fields become the densities' potentials (uniform_fields!), then residuals!."""
    kw = dict(dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), f=0.3, chi=0.3)
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    rng = np.random.default_rng(12)
    a = 0.3 + 0.05 * rng.standard_normal(o.shape)
    rho = {1: a, 2: 1.0 - a}
    for mid, r in rho.items():
        o.density[mid] = r.copy()
    o.uniform_fields()
    o.residuals_update()
    pf.fieldinit(g, rho, field_type="rho")
    for mid in (1, 2):
        assert rel(g.fields[mid], o.fields[mid]) < 1e-12
        assert rel(g.residuals[mid], o.residuals[mid]) < 1e-9


def test_scft_nsave_writes_the_fields(tmp_path):
    kw = dict(dims=(64, 1, 1), crystal="lamellar", params=(10.0,))
    g = SY.diblock_system(pf, precision="fp64", **kw)
    p = tmp_path / "ckpt.json"
    r = pf.scft(g, pf.AndersonUpdater(nhist=5), opts=pf.SCFTOptions(nsteps=3, nsave=1, ftol=1e-14, savepath=str(p)))
    assert r.nsteps == 3 and not r.converged
    d = pf.loadfields(str(p))
    assert d["grid"] == (64, 1, 1) and d["mids"] == [1, 2] and d["crystal"] == "lamellar"
    assert d["cell_params"][0] == pytest.approx(10.0, rel=1e-15) and d["field_type"] == "omega"
    for mid in (1, 2):  # saved after the last step; the final residuals! leaves the fields as they are
        assert rel(d["fields"][mid], g.fields[mid]) < 1e-12
    q = tmp_path / "never.json"
    pf.scft(g, pf.AndersonUpdater(nhist=5), opts=pf.SCFTOptions(nsteps=2, nsave=0, ftol=1e-14, savepath=str(q)))
    assert not q.exists()


def test_uniform_fields_matches_oracle():
    """uniform_fields!(sys) (system.jl:348-357) on the current densities."""
    kw = dict(dims=(32, 32, 1), crystal="hexagonal", params=(9.0,), f=0.3, chi=0.3)
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision="fp64", **kw)
    o.uniform_fields()
    pf.uniform_fields(g)
    for mid in (1, 2):
        assert rel(g.fields[mid], o.fields[mid]) < 1e-10
