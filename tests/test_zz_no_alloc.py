"""pf_propagate_noalloc: propagation for callers that cannot allocate device memory.

Such a caller -- code running inside another framework's memory pool, an allocation-free
real-time loop, or a binding that owns every device buffer -- hands the engine its own device
buffers for the propagator history and the operators; the engine keeps its internal state in
a fixed __device__ array and calls no cudaMalloc.  This test plays that caller with buffers it
holds in torch, on two calls in a row, and checks the last contour step against the FP64
oracle's propagator (src/system/mde.jl:65-81) and against pf_propagate (the entry point that
allocates its own buffers), within the parity tests' tolerances (1e-10 relative for float64
propagators, 5e-5 for float32); pf_propagate_noalloc_status then reports no timed-out wait.
The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

import pf_oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
pf = pytest.importorskip("polyfields")
from polyfields import _lib as L  # noqa: E402

TOL = {"fp64": 1e-10, "fp32": 5e-5}
DTYPE = {"fp64": (np.float64, torch.float64, L.PF_FP64), "fp32": (np.float32, torch.float32, L.PF_FP32)}


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / np.max(np.abs(b)))


def host_operators(dims, crystal, params, w, vol, b, ds, npdt):
    """LW = exp(-ds vol w / 2) and LD = exp(-ds b^2 k^2 / 6) / Ng on the half spectrum in the
    engine's [kz][kx][ky] layout (k^2 from the oracle's cell, quirk Q1 fold included)."""
    nd = sum(1 for d in dims if d > 1)
    cell = O.UnitCell(nd, crystal, *params)
    cell.setup(dims)
    ng = dims[0] * dims[1] * dims[2]
    kshape = (dims[2], dims[1], dims[0] // 2 + 1)
    lw = np.exp(-ds / 2.0 * vol * w).astype(npdt)
    ld = (np.exp(-ds * b * b / 6.0 * np.broadcast_to(cell.ksq, kshape)) / ng).astype(npdt)
    return lw, np.ascontiguousarray(ld.transpose(0, 2, 1))


def oracle_propagate(dims, crystal, params, w, q0, vol, b, ds, nsteps):
    nd = sum(1 for d in dims if d > 1)
    cell = O.UnitCell(nd, crystal, *params)
    cell.setup(dims)
    solver = O.PseudoSpectralSolver(dims)
    solver.update(w, cell.ksq, vol, b, ds)
    q, out = q0.copy(), np.empty_like(q0)
    for _ in range(nsteps):
        solver.propagate(q, out)
        q, out = out, q
    return q


CASES = [((32, 32, 32), "cubic", (7.0,), "fp64"), ((32, 32, 32), "cubic", (7.0,), "fp32"),
         ((64, 64, 1), "hexagonal", (9.0,), "fp64"), ((48, 48, 48), "cubic", (8.0,), "fp32")]


@pytest.mark.parametrize("dims,crystal,params,prec", CASES, ids=[f"{c[0][0]}x{c[0][1]}x{c[0][2]}-{c[3]}" for c in CASES])
def test_noalloc_matches_oracle_and_propagate_on_two_calls(dims, crystal, params, prec):
    npdt, tdt, code = DTYPE[prec]
    nx, ny, nz = dims
    shape = (nz, ny, nx)
    nsteps, vol, b, ds = 6, 1.0, 1.0, 0.5
    lib = L.load()
    nd = sum(1 for d in dims if d > 1)
    ref_sys = pf.FieldSystem(dims, pf.UnitCell(nd, crystal, *params), precision=prec)
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (1, 2):
        rng = np.random.default_rng(seed)
        w = 0.3 * rng.standard_normal(shape)
        q0 = 1.0 + 0.1 * rng.standard_normal(shape)
        oracle = oracle_propagate(dims, crystal, params, w, q0, vol, b, ds, nsteps)
        allocating = np.empty(shape)
        L.check(lib.pf_propagate(ref_sys._h, L.dptr(w), vol, b, ds, L.dptr(q0), L.dptr(allocating), nsteps),
                ref_sys._h)

        lw, ld = host_operators(dims, crystal, params, w, vol, b, ds, npdt)
        hist = torch.empty((nsteps + 1,) + shape, dtype=tdt, device="cuda")
        hist[0] = torch.from_numpy(q0.astype(npdt)).cuda()
        lw_d = torch.from_numpy(lw).cuda()
        ld_d = torch.from_numpy(ld).cuda()
        st = lib.pf_propagate_noalloc(nx, ny, nz, code, ctypes.c_void_p(hist.data_ptr()),
                                      ctypes.c_void_p(lw_d.data_ptr()), ctypes.c_void_p(ld_d.data_ptr()), nsteps,
                                      ctypes.c_void_p(stream))
        assert st == L.PF_OK
        assert lib.pf_propagate_noalloc_status(ctypes.c_void_p(stream)) == L.PF_OK
        got = hist[nsteps].double().cpu().numpy()
        assert rel(got, oracle) < TOL[prec], (seed, "oracle", rel(got, oracle))
        assert rel(got, allocating) < TOL[prec], (seed, "pf_propagate", rel(got, allocating))


def test_noalloc_rejects_grids_beyond_its_scratch():
    """A 128^3 float64 half spectrum (17 MB) does not fit the 16 MiB array: PF_ETOOLARGE,
    before any device work."""
    lib = L.load()
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    st = lib.pf_propagate_noalloc(128, 128, 128, L.PF_FP64, p, p, p, 4, None)
    assert st == L.PF_ETOOLARGE
    st = lib.pf_propagate_noalloc(64, 64, 64, L.PF_FP64, p, p, p, 0, None)
    assert st == L.PF_EARG
