"""GPU engine vs the FP64 oracle at the production grid sizes (through the C ABI).

The kernels behind every benchmark number are instantiated per transform length
(xy_step_kernel<T, 128, 128>, z_pipe_kernel<T, 128>, and the 96 / 64 lengths), each with its
own radix plan, scratch swizzle and group strides.  These tests pin those instantiations to
the oracle on identical seeded inputs:

* propagate! (src/system/mde.jl:65-81) for a few contour steps at 128^3, 96^3, 64^3 and a
  128 x 128 x 64 tetragonal grid, float64 (1e-10) and float32 (5e-5);
* the large blend at 128^3 (AB diblock N100 fA0.4 phi0.8 + A homopolymer N50, Ns 200, the
  benchmark's state before its first iteration): density!, stored propagators, Q, residuals!,
  free_energy, field_error and scfstress (src/species/multiblock.jl:125-295,
  src/system/system.jl:266-486) in float64 (1e-10, stress 1e-9) and float32;
* the BCC diblock at 64^3 (Ns 100) and the differentiation workload's diblock at 96^3
  (fA 0.35, Ns 200): density, Q, free energy and stress in both precisions.

Float32 tolerance: 5e-5 relative on Q, densities and the propagators (float32 rounding over
200-600 rescaled contour steps; all reductions are float64); stress 2e-3 (a difference of
nearly cancelling float32 spectra).  The oracle runs on the host's cores (~40 s for the 128^3
blend).
"""
import numpy as np
import pytest

import pf_oracle as O
import systems as SY
from polyfields import workloads as W

pf = pytest.importorskip("polyfields")

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_RTOL = 5e-5
O.FFT_WORKERS = -1


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


PROP_CASES = [((128, 128, 128), "cubic", (14.0,)), ((96, 96, 96), "cubic", (8.0,)),
              ((64, 64, 64), "cubic", (7.0,)), ((128, 128, 64), "tetragonal", (14.0, 7.5))]


@pytest.mark.parametrize("dims,crystal,params", PROP_CASES, ids=["x".join(map(str, c[0])) for c in PROP_CASES])
def test_propagate_production_sizes(dims, crystal, params):
    """update! + propagate! (mde.jl:43-81): 4 contour steps, both precisions."""
    shape = (dims[2], dims[1], dims[0])
    rng = np.random.default_rng(11)
    w = 0.3 * rng.standard_normal(shape)
    q0 = 1.0 + 0.1 * rng.standard_normal(shape)
    ocell = O.UnitCell(3, crystal, *params)
    ocell.setup(dims)
    solver = O.PseudoSpectralSolver(dims)
    solver.update(w, ocell.ksq, 1.0, 1.0, 0.5)
    q = q0.copy()
    out = np.empty(shape)
    for _ in range(4):
        solver.propagate(q, out)
        q = out.copy()
    lib = pf.load_library()
    for prec, tol in (("fp64", FP64_RTOL), ("fp32", FP32_RTOL)):
        sys = pf.FieldSystem(dims, pf.UnitCell(3, crystal, *params), precision=prec)
        got = np.empty(shape)
        st = lib.pf_propagate(sys._h, w.ctypes.data_as(pf._lib._dptr), 1.0, 1.0, 0.5,
                              q0.ctypes.data_as(pf._lib._dptr), got.ctypes.data_as(pf._lib._dptr), 4)
        pf._lib.check(st, sys._h)
        assert rel(got, q) < tol, (prec, rel(got, q))
        del sys


@pytest.fixture(scope="module")
def blend128_oracle():
    o = W.blend3d_system(O, n=128)
    ref = {"Q": [sp.Q for sp in o.species], "fhelm": o.free_energy(), "ferr": o.field_error(),
           "stress": o.scfstress(), "density": {m: o.density[m].copy() for m in (1, 2)},
           "fields": {m: o.fields[m].copy() for m in (1, 2)},
           "residuals": {m: o.residuals[m].copy() for m in (1, 2)},
           "q0": {s: o.species[0].q[s].copy() for s in (1, 67, 200)},
           "qc0": {s: o.species[0].qc[s].copy() for s in (0, 133, 199)},
           "q1": {s: o.species[1].q[s].copy() for s in (1, 100, 200)}}
    del o
    return ref


def test_blend128_fp64(blend128_oracle):
    """The benchmark's 128^3 blend at its initial state, float64 chains: every quantity of one
    residuals! + free_energy + scfstress at the FP64 bar."""
    ref = blend128_oracle
    g = W.blend3d_system(pf, n=128, precision="fp64")
    for isp in range(2):
        assert g.species[isp].Q == pytest.approx(ref["Q"][isp], rel=FP64_RTOL)
    for s, q in ref["q0"].items():
        assert rel(g.species[0].propagator(s), q) < FP64_RTOL, ("q", s)
    for s, q in ref["qc0"].items():
        assert rel(g.species[0].propagator(s, conjugate=True), q) < FP64_RTOL, ("qc", s)
    for s, q in ref["q1"].items():
        assert rel(g.species[1].propagator(s), q) < FP64_RTOL, ("homopolymer q", s)
    for mid in (1, 2):
        assert rel(g.fields[mid], ref["fields"][mid]) < FP64_RTOL
        assert rel(g.density[mid], ref["density"][mid]) < FP64_RTOL
        assert rel(g.residuals[mid], ref["residuals"][mid]) < 1e-9
    assert g.free_energy() == pytest.approx(ref["fhelm"], rel=FP64_RTOL)
    assert g.field_error() == pytest.approx(ref["ferr"], rel=1e-9)
    assert np.allclose(g.scfstress(), ref["stress"], rtol=1e-9, atol=1e-15)


def test_blend128_fp32(blend128_oracle):
    """The same state with float32 chains (the benchmark's timed path): rescaled propagators
    read back unscaled, Q, densities, free energy and stress against the oracle.

    The double-gyroid start makes Q ~ 1e47 (ln Q ~ 108): a relative error of Q is an absolute
    error of ln Q, which the 200 rescaled float32 steps of a chain accumulate step by step
    (about 4e-7 each).  Q and the unscaled propagators (whose scale is Q's) are held to 2e-4;
    the densities, in which that common scale cancels, to 5e-5."""
    ref = blend128_oracle
    g = W.blend3d_system(pf, n=128, precision="fp32")
    err = {"Q": max(abs(g.species[i].Q / ref["Q"][i] - 1) for i in range(2)),
           "q": max(rel(g.species[0].propagator(s), q) for s, q in ref["q0"].items()),
           "qc": max(rel(g.species[0].propagator(s, conjugate=True), q) for s, q in ref["qc0"].items()),
           "density": max(rel(g.density[m], ref["density"][m]) for m in (1, 2)),
           "fhelm": abs(g.free_energy() / ref["fhelm"] - 1)}
    stress = g.scfstress()
    print("float32 128^3 blend errors:", err, "stress", stress, ref["stress"])
    assert err["Q"] < 2e-4 and err["q"] < 2e-4 and err["qc"] < 2e-4, err
    assert err["density"] < FP32_RTOL, err
    assert err["fhelm"] < FP32_RTOL, err
    assert np.allclose(stress, ref["stress"], rtol=2e-3, atol=1e-9)


def _check_density_stress(o, g, tol, stress_rtol):
    assert g.species[0].Q == pytest.approx(o.species[0].Q, rel=tol)
    for mid in (1, 2):
        assert rel(g.density[mid], o.density[mid]) < tol, mid
    assert g.free_energy() == pytest.approx(o.free_energy(), rel=tol)
    assert np.allclose(g.scfstress(), o.scfstress(), rtol=stress_rtol, atol=1e-12)


@pytest.mark.parametrize("prec,tol,srtol", [("fp64", FP64_RTOL, 1e-9), ("fp32", FP32_RTOL, 2e-3)])
def test_bcc64_density_stress(prec, tol, srtol):
    """The 64^3 BCC diblock (fA 0.3, Ns 100, cubic L 7, {110} start): density and stress."""
    o = W.bcc_system(O, n=64)
    g = W.bcc_system(pf, n=64, precision=prec)
    _check_density_stress(o, g, tol, srtol)


@pytest.mark.parametrize("prec,tol,srtol", [("fp64", FP64_RTOL, 1e-9), ("fp32", FP32_RTOL, 2e-3)])
def test_diblock96_density_stress(prec, tol, srtol):
    """The differentiation workload's diblock at 96^3 (cubic L 8, fA 0.35, Ns 200)."""
    kw = dict(dims=(96, 96, 96), crystal="cubic", params=(8.0,), f=0.35, Ns=200, amp=0.3)
    o = SY.diblock_system(O, **kw)
    g = SY.diblock_system(pf, precision=prec, **kw)
    _check_density_stress(o, g, tol, srtol)
