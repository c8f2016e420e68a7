"""FP64 CPU oracle: a restatement of PolyFields.jl's SCFT hot path in NumPy.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the GPU engine is compared
against; nothing in the product path imports it.  Only the tests, the smoke check of
``__graft_entry__`` and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``
may use it.

It follows the reference's Julia sources function by function (file:line citations are
relative to the PolyFields.jl project root) including its quirks:

* Q1 k-index fold: ``ksq``/``dksq`` use |j| instead of the signed frequency
  (src/system/cell.jl:276-277, 306-307).
* Q2 stress sum: Re*Re only, every index >= 2 of the half spectrum doubled
  (src/species/multiblock.jl:279-282).
* Q3 free energy: the translational term uses phi where mu was meant
  (src/system/system.jl:407).
* Q4 dstress!: parameters restored without update!(cell) before density!
  (src/updaters/domain.jl:117-118).
* Q5 scft! reporting: ferr/fhelm evaluated on the residual of the pre-update field and
  the post-update field (src/simulate.jl:92,106-107).
* Q6 layout: dims are sorted in descending order (src/system/system.jl:58); the half
  spectrum lies on x, the fastest axis (src/utils.jl:9).

Grids are NumPy arrays of shape (Nz, Ny, Nx) in C order, i.e. x fastest, which is the
memory order of the reference's column-major ``Array{Float64,3}`` indexed [x, y, z].
Real FFTs halve the last (x) axis exactly like FFTW's r2c on the first Julia dimension.

Parity pins (checked in tests/test_oracle.py): the reference's deterministic unit tests
(test/test_cell.jl, test/test_species.jl, test/test_interactions.jl) and the converged
states it publishes (README.md:62-79, examples/examples.ipynb outputs) using the seed
files under examples/seeds.  The RNG-dependent goldens of test/test_system.jl and
test/test_updaters.jl need Julia's MersenneTwister stream and are not reproduced here.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field as dc_field
from typing import Dict, List, Optional, Sequence

import numpy as np

try:  # multi-threaded pocketfft when available
    import scipy.fft as _sfft

    def _rfftn(a, workers):
        return _sfft.rfftn(a, workers=workers)

    def _irfftn(a, shape, workers):
        return _sfft.irfftn(a, s=shape, workers=workers)
except ImportError:  # pragma: no cover
    def _rfftn(a, workers):
        return np.fft.rfftn(a)

    def _irfftn(a, shape, workers):
        return np.fft.irfftn(a, s=shape)

# Number of FFT worker threads (the reference picks min(nthreads, 1 + Ng/20000),
# src/utils.jl:16-18).  -1 = all cores.
FFT_WORKERS = 1

EPS64 = float(np.finfo(np.float64).eps)


def isapprox(a: float, b: float, rtol: float = math.sqrt(EPS64), atol: float = 0.0) -> bool:
    """Julia's default ``isapprox`` (rtol = sqrt(eps) when atol == 0)."""
    return abs(a - b) <= max(atol, rtol * max(abs(a), abs(b)))


# =============================================================================
# Basis and unit cell (src/system/basis.jl, src/system/cell.jl)
# =============================================================================
CRYSTAL1D = ("lamellar",)
CRYSTAL2D = ("square", "rectangular", "hexagonal", "oblique")
CRYSTAL3D = ("cubic", "tetragonal", "orthorhombic", "hexagonal", "monoclinic", "triclinic",
             "pnna", "fddd1")


def basis_matrix(a, b, c, alpha=math.pi / 2, beta=math.pi / 2, gamma=math.pi / 2) -> np.ndarray:
    """src/system/basis.jl:80-116.  Columns are the Bravais vectors a_i."""
    p2 = math.pi / 2
    if isapprox(alpha, p2) and isapprox(beta, p2) and isapprox(gamma, p2):
        return np.array([[a, 0.0, 0.0], [0.0, b, 0.0], [0.0, 0.0, c]], dtype=np.float64)
    cos_alpha = 0.0 if isapprox(alpha, p2) else math.cos(alpha)
    cos_beta = 0.0 if isapprox(beta, p2) else math.cos(beta)
    if isapprox(gamma, p2):
        cos_gamma, sin_gamma = 0.0, 1.0
    else:
        cos_gamma, sin_gamma = math.cos(gamma), math.sin(gamma)
    ax = a
    bx = b * cos_gamma
    by = b * sin_gamma
    cx = c * cos_beta
    cy = c * (cos_alpha - cos_beta * cos_gamma) / sin_gamma
    cz = math.sqrt(c ** 2 - cx ** 2 - cy ** 2)
    # SMat3D(ax,0,0, bx,by,0, cx,cy,cz) is column-major
    return np.array([[ax, bx, cx], [0.0, by, cy], [0.0, 0.0, cz]], dtype=np.float64)


def make_basis(dim: int, crystal: str, params: Sequence[float]) -> np.ndarray:
    """src/system/basis.jl:11-71."""
    p = list(params)
    pi = math.pi
    if dim == 1:
        if crystal not in CRYSTAL1D:
            raise ValueError(f"Unrecognized crystal system `{crystal}` for dim = {dim}.")
        assert len(p) == 1
        return basis_matrix(p[0], 1.0, 1.0, pi / 2, pi / 2, pi / 2)
    if dim == 2:
        if crystal not in CRYSTAL2D:
            raise ValueError(f"Unrecognized crystal system `{crystal}` for dim = {dim}.")
        if crystal == "square":
            assert len(p) == 1
            return basis_matrix(p[0], p[0], 1.0, pi / 2, pi / 2, pi / 2)
        if crystal == "rectangular":
            assert len(p) == 2
            return basis_matrix(p[0], p[1], 1.0, pi / 2, pi / 2, pi / 2)
        if crystal == "hexagonal":
            assert len(p) == 1
            return basis_matrix(p[0], p[0], 1.0, pi / 2, pi / 2, pi / 3)
        assert len(p) == 3  # oblique
        return basis_matrix(p[0], p[1], 1.0, pi / 2, pi / 2, p[2])
    if dim == 3:
        if crystal not in CRYSTAL3D:
            raise ValueError(f"Unrecognized crystal system `{crystal}` for dim = {dim}.")
        if crystal == "cubic":
            assert len(p) == 1
            return basis_matrix(p[0], p[0], p[0], pi / 2, pi / 2, pi / 2)
        if crystal == "tetragonal":
            assert len(p) == 2
            return basis_matrix(p[0], p[0], p[1], pi / 2, pi / 2, pi / 2)
        if crystal == "orthorhombic":
            assert len(p) == 3
            return basis_matrix(p[0], p[1], p[2], pi / 2, pi / 2, pi / 2)
        if crystal == "hexagonal":
            assert len(p) == 2
            return basis_matrix(p[0], p[0], p[1], pi / 2, pi / 2, pi / 3)
        if crystal == "monoclinic":
            assert len(p) == 4
            return basis_matrix(p[0], p[1], p[2], pi / 2, p[3], pi / 2)
        if crystal == "triclinic":
            assert len(p) == 6
            return basis_matrix(*p)
        if crystal == "pnna":
            assert len(p) == 1
            return basis_matrix(2.0 * p[0], math.sqrt(3.0) * p[0], p[0], pi / 2, pi / 2, pi / 2)
        assert len(p) == 1  # fddd1
        return basis_matrix(p[0], math.sqrt(3.0) * p[0], 2.0 * math.sqrt(3.0) * p[0],
                            pi / 2, pi / 2, pi / 2)
    raise ValueError(f"Invalid dimension {dim}")


def basis_dimensions(basis: np.ndarray) -> np.ndarray:
    """src/system/basis.jl:123-135."""
    lx, ly, lz = basis[0, 0], basis[1, 1], basis[2, 2]
    xy, xz, yz = basis[0, 1], basis[0, 2], basis[1, 2]
    a = lx
    b = math.sqrt(ly ** 2 + xy ** 2)
    c = math.sqrt(lz ** 2 + xz ** 2 + yz ** 2)
    alpha = math.acos((xy * xz + ly * yz) / (b * c))
    beta = math.acos(xz / c)
    gamma = math.acos(xy / b)
    return np.array([a, b, c, alpha, beta, gamma])


def ksize(dims):
    """src/utils.jl:9: half spectrum on the first (x) dimension."""
    return (dims[0] // 2 + 1, dims[1], dims[2])


def ndims_of(dims) -> int:
    """src/utils.jl:7."""
    return sum(1 for d in dims if d > 1)


def folded_indices(dims, signed: bool = False):
    """Folded wavevector indices jx, jy, jz on the half-spectrum grid, each broadcastable to
    shape (Nz, Ny, Kx).  src/system/cell.jl:273-277 (quirk Q1: |j| instead of signed j).  With
    signed=True the physical signed frequencies (j - N above N/2; the Nyquist index stays +N/2)
    instead, the option quirk Q1 asks to expose."""
    kx, ny, nz = ksize(dims)
    ix = np.arange(kx, dtype=np.float64)
    iy = np.arange(ny, dtype=np.float64)
    iz = np.arange(nz, dtype=np.float64)
    jy = np.where(iy <= ny / 2, iy, iy - ny if signed else ny - iy)
    jz = np.where(iz <= nz / 2, iz, iz - nz if signed else nz - iz)
    return ix[None, None, :], jy[None, :, None], jz[:, None, None]


class UnitCell:
    """src/system/cell.jl:14-109.  ``signed_k`` (default False, the reference's fold) switches
    ksq/dksq to signed frequencies (quirk Q1's option; ``set_signed_k``)."""

    signed_k = False

    def __init__(self, dim: int, crystal: str, *params):
        if len(params) == 1 and isinstance(params[0], (list, tuple, np.ndarray)):
            params = tuple(params[0])
        self.dim = int(dim)
        self.crystal = str(crystal).lstrip(":")
        self.params = np.array(params, dtype=np.float64)
        npr = self.nparams
        self.dR = np.zeros((3, 3, npr))
        self.dG = np.zeros((3, 3, npr))
        self.dRR = np.zeros((3, 3, npr))
        self.dGG = np.zeros((3, 3, npr))
        self.dims = None
        self.ksq = None
        self.dksq: List[np.ndarray] = []
        self.update()

    @property
    def nparams(self) -> int:
        return len(self.params)

    def setup(self, dims):
        """cell.jl:72-86."""
        if ndims_of(dims) != self.dim:
            raise ValueError("Number of non-singleton dimensions in System and Cell do not match!")
        self.dims = tuple(dims)
        self.ksq_update()

    def update(self):
        """cell.jl:96-109."""
        self.basis()
        self.dbasis()
        self.ddbasis()
        if self.dims is not None:
            self.ksq_update()

    def basis(self):
        """cell.jl:113-118."""
        self.R = make_basis(self.dim, self.crystal, self.params)
        self.G = 2 * math.pi * np.linalg.inv(self.R).T
        self.volume = float(np.linalg.det(self.R))

    def dbasis(self):
        """cell.jl:120-231."""
        dR = np.zeros((3, 3, self.nparams))
        c = self.crystal
        p = self.params
        if self.dim == 1:
            if c == "lamellar":
                dR[0, 0, 0] = 1.0
        elif self.dim == 2:
            if c == "square":
                dR[0, 0, 0] = 1.0
                dR[1, 1, 0] = 1.0
            elif c == "rectangular":
                dR[0, 0, 0] = 1.0
                dR[1, 1, 1] = 1.0
            elif c == "hexagonal":
                dR[0, 0, 0] = 1.0
                dR[0, 1, 0] = 0.5
                dR[1, 1, 0] = math.sqrt(0.75)
            elif c == "oblique":
                a, b, gamma = p
                dR[0, 0, 0] = 1.0
                dR[0, 1, 1] = math.cos(gamma)
                dR[1, 1, 1] = math.sin(gamma)
                dR[0, 1, 2] = -b * math.sin(gamma)
                dR[1, 1, 2] = b * math.cos(gamma)
        elif self.dim == 3:
            if c == "cubic":
                dR[0, 0, 0] = dR[1, 1, 0] = dR[2, 2, 0] = 1.0
            elif c == "tetragonal":
                dR[0, 0, 0] = dR[1, 1, 0] = 1.0
                dR[2, 2, 1] = 1.0
            elif c == "orthorhombic":
                dR[0, 0, 0] = dR[1, 1, 1] = dR[2, 2, 2] = 1.0
            elif c == "hexagonal":
                dR[0, 0, 0] = 1.0
                dR[0, 1, 0] = 0.5
                dR[1, 1, 0] = math.sqrt(0.75)
                dR[2, 2, 1] = 1.0
            elif c == "monoclinic":
                a, b, cc, beta = p
                dR[0, 0, 0] = 1.0
                dR[1, 1, 1] = 1.0
                dR[0, 2, 2] = math.cos(beta)
                dR[2, 2, 2] = math.sin(beta)
                dR[0, 2, 3] = -cc * math.sin(beta)
                dR[2, 2, 3] = cc * math.cos(beta)
            elif c == "triclinic":
                a, b, cc, alpha, beta, gamma = p
                cx, cy, cz = self.R[0, 2], self.R[1, 2], self.R[2, 2]
                sa, ca = math.sin(alpha), math.cos(alpha)
                sb, cb = math.sin(beta), math.cos(beta)
                sg, cg = math.sin(gamma), math.cos(gamma)
                tg = math.tan(gamma)
                dR[0, 0, 0] = 1.0
                dR[0, 1, 1] = cg
                dR[1, 1, 1] = sg
                dR[0, 2, 2] = cb
                dR[1, 2, 2] = cy / cc
                dR[2, 2, 2] = cz / cc
                dR[1, 2, 3] = -cc * sa / sg
                dR[2, 2, 3] = cc ** 2 * (ca - cb * cg) * sa / sg ** 2 / cz
                dR[0, 2, 4] = -cc * sb
                dR[1, 2, 4] = cc * sb / tg
                dR[2, 2, 4] = cc ** 2 * (-ca / tg + cb / sg) * sb / sg / cz
                dR[0, 1, 5] = -b * sg
                dR[1, 1, 5] = b * cg
                dR[1, 2, 5] = cc * (-ca / tg + cb / sg) / sg
                dR[2, 2, 5] = cc ** 2 * ((2 + math.cos(2 * alpha) + math.cos(2 * beta)) / tg
                                         - ca * cb * (3 + math.cos(2 * gamma)) / sg) / sg ** 2 / cz / 2
            elif c == "pnna":
                dR[0, 0, 0] = 2.0
                dR[1, 1, 0] = math.sqrt(3.0)
                dR[2, 2, 0] = 1.0
            elif c == "fddd1":
                dR[0, 0, 0] = 1.0
                dR[1, 1, 0] = math.sqrt(3.0)
                dR[2, 2, 0] = 2.0 * math.sqrt(3.0)
        self.dR = dR
        G = self.G
        dG = np.zeros((3, 3, self.nparams))
        d = self.dim
        for k in range(self.nparams):
            for i in range(d):
                for j in range(d):
                    for l in range(d):
                        for m in range(d):
                            dG[i, j, k] -= G[i, l] * dR[m, l, k] * G[m, j]
        self.dG = dG / (2 * math.pi)

    def ddbasis(self):
        """cell.jl:233-258."""
        R = self.R.T
        G = self.G
        dR, dG = self.dR, self.dG
        d = self.dim
        dRR = np.zeros((3, 3, self.nparams))
        dGG = np.zeros((3, 3, self.nparams))
        for k in range(self.nparams):
            for i in range(d):
                for j in range(d):
                    for l in range(d):
                        dRR[i, j, k] += R[i, l] * dR[l, j, k] + R[j, l] * dR[l, i, k]
                        dGG[i, j, k] += G[l, i] * dG[l, j, k] + G[l, j] * dG[l, i, k]
        self.dRR, self.dGG = dRR, dGG

    def set_signed_k(self, on: bool = True):
        self.signed_k = bool(on)
        if self.dims is not None:
            self.ksq_update()

    def ksq_update(self):
        """ksq! and dksq! (cell.jl:268-320), quirk Q1 fold included (unless signed_k)."""
        jx, jy, jz = folded_indices(self.dims, self.signed_k)
        G = self.G
        # kvec = G * jvec  (G columns are the reciprocal vectors)
        kx = G[0, 0] * jx + G[0, 1] * jy + G[0, 2] * jz
        ky = G[1, 0] * jx + G[1, 1] * jy + G[1, 2] * jz
        kz = G[2, 0] * jx + G[2, 1] * jy + G[2, 2] * jz
        self.ksq = kx * kx + ky * ky + kz * kz
        jv = (jx, jy, jz)
        self.dksq = []
        for k in range(self.nparams):
            acc = np.zeros(np.broadcast_shapes(jx.shape, jy.shape, jz.shape))
            for l in range(self.dim):
                for m in range(self.dim):
                    acc = acc + jv[l] * jv[m] * self.dGG[l, m, k]
            self.dksq.append(acc)


# =============================================================================
# Monomers, species, interactions
# =============================================================================
@dataclass(frozen=True)
class Monomer:
    """src/system/monomer.jl:7-25."""
    id: int
    vol: float = 1.0
    charge: float = 0.0


def chain_grid(N_block: Sequence[float], Ns: int):
    """src/species/base.jl:27-56."""
    N = float(sum(N_block))
    nblocks = len(N_block)
    ds = N / Ns
    begin_block = [0] * (nblocks + 1)
    ds_block = [0.0] * nblocks
    bgn = 1
    begin_block[0] = bgn
    for iblk in range(nblocks):
        Ns_half = int(math.floor(N_block[iblk] / ds / 2.0 + 0.5))
        if Ns_half == 0:
            Ns_half = 1
            ds_block[iblk] = N_block[iblk] / 2.0
        else:
            ds_block[iblk] = N_block[iblk] / Ns_half / 2.0
        bgn = bgn + Ns_half * 2
        begin_block[iblk + 1] = bgn
    return N, begin_block, ds_block


class Multiblock:
    """src/species/multiblock.jl:5-77.  ``begin_block`` keeps Julia's 1-based contour
    indices; ``q[s-1]`` is the reference's ``q[s]``."""

    def __init__(self, mon_block: Sequence[Monomer], N_block: Sequence[int],
                 b_block: Sequence[float], Ns: int = 100):
        assert len(mon_block) == len(N_block) == len(b_block)
        self.monomers = sorted(set(mon_block), key=lambda m: m.id)
        self.mids = [m.id for m in self.monomers]
        self.mid_block = [m.id for m in mon_block]
        self.mid_map: Dict[int, List[int]] = {}
        for iblk, mid in enumerate(self.mid_block):
            self.mid_map.setdefault(mid, []).append(iblk)
        self.N = int(sum(N_block))
        self.N_block = [int(n) for n in N_block]
        self.Nref_block = [mon_block[i].vol * N_block[i] for i in range(len(mon_block))]
        self.Nref, self.begin_block, self.ds_block = chain_grid(self.Nref_block, Ns)
        self.f_block = [nr / self.Nref for nr in self.Nref_block]
        self.b_block = [float(b) for b in b_block]
        if Ns != self.begin_block[-1] - 1:
            Ns = self.begin_block[-1] - 1  # multiblock.jl:56-59 (warning in the reference)
        self.Ns = Ns
        self.Q = 0.0
        self.q: List[np.ndarray] = []
        self.qc: List[np.ndarray] = []
        self.density: Dict[int, np.ndarray] = {}
        self.density_block: Dict[int, np.ndarray] = {}
        self.system = None

    @property
    def nblocks(self):
        return len(self.N_block)

    def hasmonomer(self, mid):
        return mid in self.mids

    def monomer_fraction(self, mid):
        """multiblock.jl:93-102."""
        if not self.hasmonomer(mid):
            return 0.0
        return sum(self.f_block[i] for i in self.mid_map[mid])

    def setup(self, sys):
        """multiblock.jl:104-121."""
        self.system = sys
        self.Q = 0.0
        self.q = [np.zeros(sys.shape) for _ in range(self.Ns + 1)]
        self.qc = [np.zeros(sys.shape) for _ in range(self.Ns + 1)]
        for mid in self.mids:
            self.density[mid] = np.zeros(sys.shape)
        for iblk in range(self.nblocks):
            self.density_block[iblk] = np.zeros(sys.shape)

    def density_update(self):
        """density!(chain) — multiblock.jl:125-231."""
        sys = self.system
        q, qc = self.q, self.qc
        solver = sys.solver
        ksq = sys.cell.ksq
        q[0][...] = 1.0
        for iblk in range(self.nblocks):
            mon = sys.monomers[self.mid_block[iblk]]
            solver.update(sys.fields[mon.id], ksq, mon.vol, self.b_block[iblk], self.ds_block[iblk])
            for s in range(self.begin_block[iblk], self.begin_block[iblk + 1]):
                solver.propagate(q[s - 1], q[s])
        if self.nblocks == 1:
            for s, qi in enumerate(reversed(q)):
                qc[s][...] = qi
        else:
            qc[-1][...] = 1.0
            for iblk in range(self.nblocks - 1, -1, -1):
                mon = sys.monomers[self.mid_block[iblk]]
                solver.update(sys.fields[mon.id], ksq, mon.vol, self.b_block[iblk],
                              self.ds_block[iblk])
                for s in range(self.begin_block[iblk + 1], self.begin_block[iblk], -1):
                    solver.propagate(qc[s - 1], qc[s - 2])
        self.Q = float(np.sum(q[-1])) / sys.ngrid
        for rho in self.density.values():
            rho[...] = 0.0
        for iblk in range(self.nblocks):
            bgn, end = self.begin_block[iblk], self.begin_block[iblk + 1]
            ds = self.ds_block[iblk]
            rho = np.zeros(sys.shape)
            rho += q[bgn - 1] * qc[bgn - 1]
            rho += q[end - 1] * qc[end - 1]
            for s in range(bgn + 1, end, 2):
                rho += 4.0 * q[s - 1] * qc[s - 1]
            for s in range(bgn + 2, end - 1, 2):
                rho += 2.0 * q[s - 1] * qc[s - 1]
            rho *= ds / 3.0
            self.density_block[iblk] = rho
        for iblk in range(self.nblocks):
            self.density_block[iblk] /= self.Q * self.Nref
        for mid in self.mids:
            for iblk in self.mid_map[mid]:
                self.density[mid] += self.density_block[iblk]

    def scfstress(self):
        """multiblock.jl:233-295 (quirk Q2)."""
        sys = self.system
        cell = sys.cell
        q, qc = self.q, self.qc
        dQ = np.zeros(cell.nparams)
        ng = sys.ngrid
        for iblk in range(self.nblocks):
            bgn, end = self.begin_block[iblk], self.begin_block[iblk + 1]
            b = self.b_block[iblk]
            ds0 = self.ds_block[iblk]
            for s in range(bgn, end + 1):
                ds = ds0
                if s != bgn and s != end:
                    ds *= 4.0 if s % 2 == 0 else 2.0
                qk1 = _rfftn(q[s - 1], FFT_WORKERS).ravel()
                qk2 = _rfftn(qc[s - 1], FFT_WORKERS).ravel()
                for k in range(cell.nparams):
                    dk = np.broadcast_to(cell.dksq[k], sys.kshape).ravel()
                    tmp_re = qk1.real * dk
                    qint = qk2.real[0] * tmp_re[0] + 2.0 * float(np.dot(qk2.real[1:], tmp_re[1:]))
                    dQ[k] -= b ** 2 * ds * qint / 6.0 / ng ** 2
        dQ /= 3.0
        dQ /= self.Q * self.Nref
        return dQ


def Homopolymer(mon: Monomer, N: int, b: float, Ns: int = 100) -> Multiblock:
    """multiblock.jl:62-64."""
    return Multiblock([mon], [N], [b], Ns)


def Diblock(amon: Monomer, bmon: Monomer, N: int, f: float, b1: float, b2: float,
            Ns: int = 100) -> Multiblock:
    """multiblock.jl:66-72: block lengths truncated to integers; error when they do not sum
    to N."""
    N_block = [int(f * N), int((1 - f) * N)]  # trunc.(Int, ...)
    if sum(N_block) != N:
        raise ValueError(f"Non-integer block lengths for N = {N}, f = {f}.")
    return Multiblock([amon, bmon], N_block, [b1, b2], Ns)


class Point:
    """src/species/point.jl:9-58."""

    def __init__(self, mon: Monomer):
        self.mids = [mon.id]
        self.Nref = mon.vol
        self.Q = 0.0
        self.density: Dict[int, np.ndarray] = {}
        self.system = None

    def hasmonomer(self, mid):
        return mid in self.mids

    def monomer_fraction(self, mid):
        return 1.0 if self.hasmonomer(mid) else 0.0

    def setup(self, sys):
        self.system = sys
        self.Q = 0.0
        self.density[self.mids[0]] = np.zeros(sys.shape)

    def density_update(self):
        sys = self.system
        mon = sys.monomers[self.mids[0]]
        omega = sys.fields[mon.id]
        boltz = np.exp(-mon.vol * omega)
        self.Q = float(np.sum(boltz)) / sys.ngrid
        self.density[mon.id] = boltz / self.Q

    def scfstress(self):
        return np.zeros(self.system.cell.nparams)


class FloryInteraction:
    """src/interactions/flory.jl:9-100."""

    def __init__(self):
        self.mids = set()
        self.chis: Dict[tuple, float] = {}
        self.system = None

    def set_interaction(self, alpha, beta, chi):
        if isinstance(alpha, Monomer):
            alpha = alpha.id
        if isinstance(beta, Monomer):
            beta = beta.id
        assert alpha != beta
        pair = (alpha, beta) if alpha <= beta else (beta, alpha)
        self.mids.add(alpha)
        self.mids.add(beta)
        self.chis[pair] = float(chi)

    def setup(self, sys):
        self.system = sys

    def energy(self):
        sys = self.system
        e = 0.0
        for (a, b), chi in self.chis.items():
            if a in sys.monomers and b in sys.monomers:
                va, vb = sys.monomers[a].vol, sys.monomers[b].vol
                e += float(np.sum(chi * (sys.density[a] / va) * (sys.density[b] / vb)))
        return e / sys.ngrid

    def energy_bulk(self):
        sys = self.system
        e = 0.0
        for (a, b), chi in self.chis.items():
            if a in sys.monomers and b in sys.monomers:
                va, vb = sys.monomers[a].vol, sys.monomers[b].vol
                e += chi * (sys.monomer_fracs[a] / va) * (sys.monomer_fracs[b] / vb)
        return e

    def potential(self, alpha, pot):
        sys = self.system
        for beta in sorted(self.mids):
            pair = (alpha, beta) if alpha <= beta else (beta, alpha)
            if pair not in self.chis:
                continue
            chi = self.chis[pair]
            pot += chi * (sys.density[beta] / sys.monomers[beta].vol)


class EdwardsInteraction:
    """src/interactions/edwards.jl:9-87."""

    def __init__(self):
        self.mids = set()
        self.uvals: Dict[int, float] = {}
        self.system = None

    def set_interaction(self, mid, u):
        if isinstance(mid, Monomer):
            mid = mid.id
        self.mids.add(mid)
        self.uvals[mid] = float(u)

    def setup(self, sys):
        self.system = sys

    def energy(self):
        sys = self.system
        e = 0.0
        for mid in self.mids:
            if mid in sys.monomers:
                u, v = self.uvals[mid], sys.monomers[mid].vol
                e += float(np.sum((u / 2) * (sys.density[mid] / v) ** 2))
        return e / sys.ngrid

    def energy_bulk(self):
        sys = self.system
        e = 0.0
        for mid in self.mids:
            if mid in sys.monomers:
                u, v = self.uvals[mid], sys.monomers[mid].vol
                e += (u / 2) * (sys.monomer_fracs[mid] / v) ** 2
        return e

    def potential(self, mid, pot):
        sys = self.system
        if mid in self.mids:
            pot += self.uvals[mid] * (sys.density[mid] / sys.monomers[mid].vol)


# =============================================================================
# MDE solver (src/system/mde.jl)
# =============================================================================
class PseudoSpectralSolver:
    """src/system/mde.jl:7-106 with the FFTHolder of src/system/fft.jl."""

    def __init__(self, dims, method: str = "RK2"):
        if method not in ("RK2", "RQM4"):
            raise ValueError(f"Invalid propagator method `{method}` for PseudoSpectralSolver.")
        self.dims = tuple(dims)
        self.method = method
        self.shape = (dims[2], dims[1], dims[0])
        self.LW1 = self.LW2 = self.LD1 = self.LD2 = None

    def update(self, omega, ksq, vol, b, ds):
        """mde.jl:43-57."""
        lw_coeff = ds / 2.0
        ld_coeff = ds * b ** 2 / 6.0
        self.LW1 = np.exp(-lw_coeff * vol * omega)
        self.LW2 = np.exp(-lw_coeff * vol * omega / 2.0)
        self.LD1 = np.exp(-ld_coeff * ksq)
        self.LD2 = np.exp(-ld_coeff * ksq / 2.0)

    def _ft(self, a):
        return _rfftn(a, FFT_WORKERS)

    def _ift(self, a):
        return _irfftn(a, self.shape, FFT_WORKERS)

    def propagate(self, qin, qout):
        """mde.jl:65-104."""
        LW1, LW2, LD1, LD2 = self.LW1, self.LW2, self.LD1, self.LD2
        if self.method == "RK2":
            qr = LW1 * qin
            qk = self._ft(qr) * LD1
            qr = self._ift(qk)
            qout[...] = LW1 * qr
        else:
            qr = LW1 * qin
            qk = self._ft(qr) * LD1
            q1 = LW1 * self._ift(qk)
            qr = LW2 * qin
            qk = self._ft(qr) * LD2
            qr = self._ift(qk) * LW1
            qk = self._ft(qr) * LD2
            q2 = LW2 * self._ift(qk)
            qout[...] = (4.0 * q2 - q1) / 3.0


# =============================================================================
# Field system (src/system/system.jl, src/system/compress.jl)
# =============================================================================
CANONICAL = "Canonical"
GRAND = "Grand"


class Compressibility:
    """src/system/compress.jl:7-61."""

    def __init__(self, inv_zeta: float = 0.0):
        self.inv_zeta = float(inv_zeta)
        self.strict = isapprox(inv_zeta, 0.0, atol=0.0) if inv_zeta != 0.0 else True
        self.field = None
        self.system = None

    def setup(self, sys):
        self.system = sys
        self.field = np.zeros(sys.shape)

    def update(self):
        sys = self.system
        rhosum = np.zeros(sys.shape)
        for mid in sys.monomers:
            rhosum += sys.density[mid]
        self.field = np.zeros(sys.shape)
        if self.strict:
            f = rhosum - 1.0
            for mid in sys.monomers:
                f += sys.fields[mid] - sys.potentials[mid]
            self.field = f / len(sys.monomers)
        elif self.inv_zeta > 0.0:
            self.field = (1.0 / self.inv_zeta) * (rhosum - 1.0)


class FieldSystem:
    """src/system/system.jl:22-76."""

    def __init__(self, dims, cell: UnitCell, monomers: Sequence[Monomer] = (),
                 ensemble: str = CANONICAL, compress: Optional[Compressibility] = None,
                 mde: str = "RK2"):
        dims = tuple(int(d) for d in dims)
        sdims = tuple(sorted(dims, reverse=True))
        if sdims != dims:
            # the reference builds FFT plans and solver grids with the unsorted dims
            # (system.jl:55-58) and then fails on the first size assertion
            raise AssertionError("dims must be given in descending order")
        self.dims = sdims
        self.shape = (sdims[2], sdims[1], sdims[0])
        self.kshape = (sdims[2], sdims[1], sdims[0] // 2 + 1)
        self.ensemble = ensemble
        self.cell = cell
        self.solver = PseudoSpectralSolver(sdims, method=mde)
        self.monomers: Dict[int, Monomer] = {}
        self.monomer_fracs: Dict[int, float] = {}
        self.fields: Dict[int, np.ndarray] = {}
        self.potentials: Dict[int, np.ndarray] = {}
        self.residuals: Dict[int, np.ndarray] = {}
        self.density: Dict[int, np.ndarray] = {}
        self.interactions = []
        self.species = []
        self.phi_species: List[float] = []
        self.mu_species: List[float] = []
        self.compress = compress if compress is not None else Compressibility(0.0)
        cell.setup(sdims)
        self.compress.setup(self)
        for mon in monomers:
            self.add_monomer(mon)

    @property
    def ngrid(self):
        return self.dims[0] * self.dims[1] * self.dims[2]

    def volume(self):
        return self.cell.volume

    def add_cell(self, cell):
        self.cell = cell
        cell.setup(self.dims)

    def add_monomer(self, mon: Monomer):
        self.monomers[mon.id] = mon
        self.monomer_fracs[mon.id] = 0.0
        self.fields[mon.id] = np.zeros(self.shape)
        self.potentials[mon.id] = np.zeros(self.shape)
        self.residuals[mon.id] = np.zeros(self.shape)
        self.density[mon.id] = np.zeros(self.shape)

    def add_species(self, species, val: float):
        """system.jl:137-161."""
        for mid in species.mids:
            if mid not in self.monomers:
                raise ValueError(f"Species contains monomer with id = {mid} not present in system.")
        species.setup(self)
        self.species.append(species)
        if self.ensemble == CANONICAL:
            if val <= 0.0:
                raise ValueError("Bulk volume fraction must be 0 < phi <= 1.")
            self.phi_species.append(float(val))
            self.mu_species.append(0.0)
        else:
            self.phi_species.append(0.0)
            self.mu_species.append(float(val))

    def add_interaction(self, itx):
        for mid in itx.mids:
            if mid not in self.monomers:
                raise ValueError(f"Interaction contains monomer with id = {mid} not present in system.")
        itx.setup(self)
        self.interactions.append(itx)

    def validate(self):
        """system.jl:192-237."""
        if not any(float(np.mean(w)) != 0.0 or float(np.std(w)) != 0.0 for w in self.fields.values()):
            raise ValueError("Fields must be initialized before SCFT simulation.")
        if self.ensemble == CANONICAL and not isapprox(sum(self.phi_species), 1.0):
            raise ValueError("Species volume fractions do not sum to unity.")
        self.monomer_fractions()
        bulk_charge = sum(self.monomer_fracs[mid] * m.charge / m.vol for mid, m in self.monomers.items())
        if not isapprox(bulk_charge, 0.0):
            raise ValueError("Bulk system not charge neutral.")
        for mid in self.monomers:
            if not any(sp.hasmonomer(mid) for sp in self.species):
                raise ValueError(f"Monomer with ID = {mid} not found in any species.")

    def muphi(self):
        """system.jl:248-259."""
        for isp, sp in enumerate(self.species):
            if self.ensemble == CANONICAL:
                self.mu_species[isp] = math.log(self.phi_species[isp] / sp.Q)
            else:
                self.phi_species[isp] = sp.Q * math.exp(self.mu_species[isp])

    def density_update(self):
        """density!(sys) — system.jl:266-289."""
        for mid in self.density:
            self.density[mid] = np.zeros(self.shape)
        for sp in self.species:
            sp.density_update()
        self.muphi()
        for isp, sp in enumerate(self.species):
            phi = self.phi_species[isp]
            for mid in sp.mids:
                self.density[mid] += phi * sp.density[mid]

    def potentials_update(self):
        """system.jl:296-310."""
        for mid in self.potentials:
            pot = np.zeros(self.shape)
            for itx in self.interactions:
                itx.potential(mid, pot)
            self.potentials[mid] = pot

    def residuals_update(self):
        """residuals!(sys) — system.jl:317-340."""
        self.density_update()
        self.potentials_update()
        self.compress.update()
        eta = self.compress.field
        for mid in self.residuals:
            self.residuals[mid] = self.potentials[mid] + eta - self.fields[mid]
        if self.ensemble == CANONICAL:
            for mid in self.fields:
                self.fields[mid] -= np.mean(self.fields[mid])
                self.residuals[mid] -= np.mean(self.residuals[mid])

    def uniform_fields(self):
        """system.jl:348-357."""
        self.potentials_update()
        for mid in self.fields:
            self.fields[mid] = self.potentials[mid].copy()
            if self.ensemble == CANONICAL:
                self.fields[mid] -= np.mean(self.fields[mid])

    def monomer_fractions(self):
        """system.jl:364-375."""
        for mid in self.monomer_fracs:
            self.monomer_fracs[mid] = 0.0
        for isp, sp in enumerate(self.species):
            for mid in sp.mids:
                self.monomer_fracs[mid] += self.phi_species[isp] * sp.monomer_fraction(mid)
        return self.monomer_fracs

    def scfstress(self):
        """system.jl:384-395."""
        stress = np.zeros(self.cell.nparams)
        self.muphi()
        for isp, sp in enumerate(self.species):
            stress -= self.phi_species[isp] * sp.scfstress()
        return stress

    def free_energy(self):
        """system.jl:402-433 (quirk Q3: mu = phi)."""
        ftrans = 0.0
        for isp, sp in enumerate(self.species):
            phi = self.phi_species[isp]
            mu = self.phi_species[isp]
            if phi > 1e-8:
                ftrans += phi * (mu - 1.0) / sp.Nref
        ffield = 0.0
        for mid, omega in self.fields.items():
            ffield -= float(np.sum(self.density[mid] * omega))
        ffield /= self.ngrid
        fexc = sum(itx.energy() for itx in self.interactions)
        return ftrans + ffield + fexc

    def free_energy_bulk(self):
        """system.jl:440-458."""
        f = 0.0
        for isp, sp in enumerate(self.species):
            phi = self.phi_species[isp]
            if phi > 1e-8:
                f += phi * (math.log(phi) - 1.0) / sp.Nref
        self.monomer_fractions()
        for itx in self.interactions:
            f += itx.energy_bulk()
        return f

    def field_error(self):
        """system.jl:470-486."""
        rsum = sum(float(np.sum(r * r)) for r in self.residuals.values())
        wsum = EPS64 + sum(float(np.sum(w * w)) for w in self.fields.values())
        return math.sqrt(rsum) / math.sqrt(wsum)


# =============================================================================
# Field updaters (src/updaters/*.jl)
# =============================================================================
def lu_inverse(A: np.ndarray) -> np.ndarray:
    """LU with partial pivoting followed by an explicit inverse, the ``inv!(lu!(A))`` of
    src/updaters/anderson.jl:185.  Raises ``np.linalg.LinAlgError`` on an exactly zero pivot
    (LAPACK getrf info > 0, Julia's SingularException)."""
    n = A.shape[0]
    a = A.astype(np.float64).copy()
    perm = list(range(n))
    for k in range(n):
        p = k + int(np.argmax(np.abs(a[k:, k])))
        if a[p, k] == 0.0:
            raise np.linalg.LinAlgError(f"SingularException({k + 1})")
        if p != k:
            a[[k, p], :] = a[[p, k], :]
            perm[k], perm[p] = perm[p], perm[k]
        a[k + 1:, k] /= a[k, k]
        a[k + 1:, k + 1:] -= np.outer(a[k + 1:, k], a[k, k + 1:])
    # solve A X = I via the factors
    inv = np.zeros((n, n))
    for col in range(n):
        e = np.zeros(n)
        e[perm.index(col)] = 1.0
        y = np.zeros(n)
        for i in range(n):
            y[i] = e[i] - np.dot(a[i, :i], y[:i])
        x = np.zeros(n)
        for i in range(n - 1, -1, -1):
            x[i] = (y[i] - np.dot(a[i, i + 1:], x[i + 1:])) / a[i, i]
        inv[:, col] = x
    return inv


class AndersonUpdater:
    """src/updaters/anderson.jl:13-228."""

    def __init__(self, nhist: int = 50, iter_euler: int = 1, lam_euler: float = 0.01):
        if iter_euler <= 1:
            iter_euler = 1
        self.nhist = int(nhist)
        self.iter = 0
        self.iter_hist = 0
        self.iter_euler = iter_euler
        self.lam = 0.0
        self.lam_euler = float(lam_euler)
        self.is_setup = False
        self.res_hist: List[Dict[int, np.ndarray]] = [dict() for _ in range(self.nhist + 1)]
        self.field_hist: List[Dict[int, np.ndarray]] = [dict() for _ in range(self.nhist + 1)]
        self.Cn = np.zeros(0)
        self.system = None

    def setup(self, sys):
        self.system = sys
        if self.is_setup:
            return
        if sys.ensemble != CANONICAL:
            raise ValueError("Anderson mixing can only be used for systems in the canonical ensemble.")
        for d in self.res_hist:
            for mid in sys.residuals:
                d[mid] = np.zeros(sys.shape)
        for d in self.field_hist:
            for mid in sys.fields:
                d[mid] = np.zeros(sys.shape)
        for mid, omega in sys.fields.items():
            self.field_hist[0][mid] = omega.copy()
        self.iter = 0
        self.iter_hist = 0
        self.lam = 0.0
        self.is_setup = True

    def step(self):
        sys = self.system
        self.iter += 1
        if self.iter < self.nhist + 1:
            self.iter_hist = self.iter - 1
            self.lam = 1.0 - 0.9 ** self.iter
        else:
            self.iter_hist = self.nhist
            self.lam = 1.0
        it, ih = self.iter, self.iter_hist
        sys.residuals_update()
        for mid, res in sys.residuals.items():
            self.res_hist[ih][mid] = res.copy()
        if it <= self.iter_euler:
            for mid in sys.fields:
                sys.fields[mid] = sys.fields[mid] + self.lam_euler * sys.residuals[mid]
        else:
            Umn = np.zeros((ih, ih))
            Vm = np.zeros(ih)
            res_iter = self.res_hist[ih]
            field_iter = self.field_hist[ih]
            for mm in range(1, ih + 1):
                res_mm = self.res_hist[ih - mm]
                for nn in range(mm, ih + 1):
                    res_nn = self.res_hist[ih - nn]
                    for mid, res in res_iter.items():
                        Umn[mm - 1, nn - 1] += float(np.sum((res - res_mm[mid]) * (res - res_nn[mid])))
                    Umn[nn - 1, mm - 1] = Umn[mm - 1, nn - 1]
                for mid, res in res_iter.items():
                    Vm[mm - 1] += float(np.sum((res - res_mm[mid]) * res))
            self.Umn, self.Vm = Umn.copy(), Vm.copy()
            try:
                inv = lu_inverse(Umn)
            except np.linalg.LinAlgError as err:
                raise RuntimeError(f"Error inverting Umn matrix on iteration {it}: {err}")
            self.Cn = inv @ Vm
            for mid in sys.fields:
                WW = sys.fields[mid].copy()
                DD = res_iter[mid].copy()
                for nn in range(1, ih + 1):
                    WW += self.Cn[nn - 1] * (self.field_hist[ih - nn][mid] - field_iter[mid])
                    DD += self.Cn[nn - 1] * (self.res_hist[ih - nn][mid] - res_iter[mid])
                sys.fields[mid] = WW + self.lam * DD
        if it < self.nhist + 1:
            for mid, omega in sys.fields.items():
                self.field_hist[it][mid] = omega.copy()
        else:
            for nh in range(self.nhist):
                for mid in sys.fields:
                    self.res_hist[nh][mid] = self.res_hist[nh + 1][mid].copy()
                    self.field_hist[nh][mid] = self.field_hist[nh + 1][mid].copy()
            for mid, omega in sys.fields.items():
                self.field_hist[-1][mid] = omega.copy()


class EulerUpdater:
    """src/updaters/euler.jl:9-65."""

    def __init__(self, method: str = "PECE", lam: float = 0.05):
        if method not in ("PEC", "PECE"):
            raise ValueError("Invalid `method` parameter for EulerUpdater. Options include: (:PEC, :PECE)")
        self.method = method
        self.lam = float(lam)
        self.fields: Dict[int, np.ndarray] = {}
        self.system = None

    def setup(self, sys):
        self.system = sys
        self.fields = {mid: w.copy() for mid, w in sys.fields.items()}

    def step(self):
        sys = self.system
        for mid in sys.fields:
            sys.fields[mid] = sys.fields[mid] + self.lam * sys.residuals[mid]
            self.fields[mid] = sys.fields[mid] + 0.5 * self.lam * sys.residuals[mid]
        sys.residuals_update()
        for mid in self.fields:
            self.fields[mid] = self.fields[mid] + 0.5 * self.lam * sys.residuals[mid]
        for mid in self.fields:
            sys.fields[mid] = self.fields[mid].copy()
        if self.method == "PECE":
            sys.residuals_update()


class MomentumUpdater:
    """src/updaters/momentum.jl:19-165: MOM (first-moment average with beta1), RMS (second
    moment with beta2, step r / (sqrt(v) + 1e-8)), ADAM (both, no bias correction) and NAG
    (look-ahead gradient with gamma); every method ends with w += lam * step."""

    def __init__(self, method: str = "MOM", lam: float = 0.01, gamma: float = 0.9, beta1: float = 0.9,
                 beta2: float = 0.999):
        assert 0.0 < gamma < 1.0 and 0.0 < beta1 < 1.0 and 0.0 < beta2 < 1.0
        if method not in ("MOM", "RMS", "ADAM", "NAG"):
            raise ValueError("Invalid `method` parameter for MomentumUpdater. Options include: (:MOM, :RMS, :ADAM, :NAG)")
        self.method = method
        self.lam, self.gamma, self.beta1, self.beta2 = float(lam), float(gamma), float(beta1), float(beta2)
        self.system = None

    def setup(self, sys):
        self.system = sys
        self.stepv = {mid: r.copy() for mid, r in sys.residuals.items()}
        self.temp = {mid: w.copy() for mid, w in sys.fields.items()}
        self.mt = {mid: np.zeros(sys.shape) for mid in sys.fields}
        self.vt = {mid: np.zeros(sys.shape) for mid in sys.fields}

    def step(self):
        sys = self.system
        b1, b2, g = self.beta1, self.beta2, self.gamma
        if self.method == "MOM":
            sys.residuals_update()
            for mid in self.mt:
                self.mt[mid] = b1 * self.mt[mid] + (1 - b1) * sys.residuals[mid]
            self.stepv = {mid: m.copy() for mid, m in self.mt.items()}
        elif self.method == "RMS":
            sys.residuals_update()
            for mid in self.vt:
                self.vt[mid] = b2 * self.vt[mid] + (1 - b2) * sys.residuals[mid] ** 2
            for mid in self.stepv:
                self.stepv[mid] = sys.residuals[mid] / (np.sqrt(self.vt[mid]) + 1e-8)
        elif self.method == "ADAM":
            sys.residuals_update()
            for mid in self.mt:
                self.mt[mid] = b1 * self.mt[mid] + (1 - b1) * sys.residuals[mid]
            for mid in self.vt:
                self.vt[mid] = b2 * self.vt[mid] + (1 - b2) * sys.residuals[mid] ** 2
            for mid in self.stepv:
                self.stepv[mid] = self.mt[mid] / (np.sqrt(self.vt[mid]) + 1e-8)
        else:  # NAG
            self.temp = {mid: w.copy() for mid, w in sys.fields.items()}
            for mid in sys.fields:
                sys.fields[mid] = sys.fields[mid] + self.lam * self.mt[mid]
            sys.residuals_update()
            for mid in self.mt:
                self.mt[mid] = g * self.mt[mid] + (1 - g) * sys.residuals[mid]
            self.stepv = {mid: m.copy() for mid, m in self.mt.items()}
            for mid in sys.fields:
                sys.fields[mid] = self.temp[mid].copy()
        for mid in sys.fields:
            sys.fields[mid] = sys.fields[mid] + self.lam * self.stepv[mid]


class DomainUpdater:
    """src/updaters/domain.jl:7-121 (quirk Q4)."""

    def __init__(self, nper: int = 10, nskip: int = 200, lam: float = 0.1, pmax: float = 1.0,
                 rlxn: float = 0.5):
        self.nper, self.nskip = int(nper), int(nskip)
        self.lam, self.pmax, self.rlxn = float(lam), float(pmax), float(rlxn)
        self.system = None

    def stress_error(self):
        return float(np.linalg.norm(self.stress))

    def setup(self, sys):
        self.system = sys
        npr = sys.cell.nparams
        self.stress = sys.scfstress()
        self.oldparams = np.zeros(npr)
        self.step_vec = np.zeros(npr)
        self.dstress = np.zeros((npr, npr))

    def scfstress_update(self):
        self.stress = self.system.scfstress()

    def step(self, nsteps: int = 1, tol: float = 1e-5):
        sys = self.system
        cell = sys.cell
        self.scfstress_update()
        it = 0
        while it < nsteps:
            self.dstress_update()
            if cell.dim == 1:
                self.step_vec = np.full(cell.nparams, -1.0 * self.stress[0] / self.dstress[0, 0])
            else:
                self.step_vec = np.linalg.inv(self.dstress) @ self.stress
                self.step_vec *= -1.0
            step_size = float(np.linalg.norm(self.step_vec))
            if step_size > self.pmax:
                self.step_vec *= self.pmax / step_size
            cell.params = cell.params + self.lam * self.step_vec
            cell.params = self.rlxn * cell.params + (1 - self.rlxn) * self.oldparams
            cell.update()
            sys.density_update()
            sys.residuals_update()
            self.scfstress_update()
            it += 1

    def dstress_update(self):
        sys = self.system
        cell = sys.cell
        self.oldparams = cell.params.copy()
        dx = 1e-8
        x = 1.0 / dx
        for k in range(cell.nparams):
            cell.params = self.oldparams.copy()
            cell.params[k] += dx
            cell.update()
            sys.density_update()
            pstress = sys.scfstress()
            self.dstress[:, k] = x * (pstress - self.stress)
        cell.params = self.oldparams.copy()
        sys.density_update()  # quirk Q4: ksq still from the perturbed parameters


# =============================================================================
# Driver (src/simulate.jl, src/fileio.jl)
# =============================================================================
@dataclass
class SCFTOptions:
    """simulate.jl:12-19."""
    nsteps: int = 100
    nsout: int = 0
    nsave: int = 0
    ftol: float = 1e-5
    stol: float = 1e-4
    savepath: str = ""


@dataclass
class SCFTResults:
    """simulate.jl:26-33."""
    time: float
    nsteps: int
    converged: bool
    ferr: float
    serr: float
    fhelm: float
    history: list = dc_field(default_factory=list)


def isconverged(ferr, ftol, serr, stol, vcell=False):
    """simulate.jl:37-49."""
    fconverged = False
    sconverged = True
    if ferr < ftol:
        fconverged = True
        if vcell and serr > stol:
            sconverged = False
    return fconverged and sconverged


def scft(sys: FieldSystem, updater, domain: Optional[DomainUpdater] = None,
         opts: Optional[SCFTOptions] = None, verbose: bool = False) -> SCFTResults:
    """scft! — simulate.jl:60-148 (quirk Q5).  ``history`` records (step, ferr, fhelm)."""
    opts = opts or SCFTOptions()
    t0 = time.perf_counter()
    sys.validate()
    sys.residuals_update()
    updater.setup(sys)
    step = 0
    ferr = sys.field_error()
    fhelm = sys.free_energy()
    serr = 0.0
    vcell = domain is not None
    if vcell:
        domain.setup(sys)
        serr = domain.stress_error()
    history = []
    converged = isconverged(ferr, opts.ftol, serr, opts.stol, vcell)
    while step < opts.nsteps and not converged:
        if verbose and opts.nsout > 0 and step % opts.nsout == 0:
            print(f"Step ({step:<5d} / {opts.nsteps:5d}): ferr = {ferr:8e}, fhelm = {fhelm:.5e}")
        updater.step()
        if vcell and step % domain.nskip == 0:
            domain.scfstress_update()
            serr = domain.stress_error()
            if serr > opts.stol:
                domain.step(nsteps=domain.nper, tol=opts.stol)
                serr = domain.stress_error()
        ferr = sys.field_error()
        fhelm = sys.free_energy()
        history.append((step, ferr, fhelm))
        if math.isnan(ferr):
            raise RuntimeError("Diverging field updater -- breaking.")
        converged = isconverged(ferr, opts.ftol, serr, opts.stol, vcell)
        if converged:
            break
        step += 1
    sys.residuals_update()
    ferr = sys.field_error()
    fhelm = sys.free_energy()
    if vcell:
        serr = domain.stress_error()
    return SCFTResults(time.perf_counter() - t0, step, converged, ferr, serr, fhelm, history)


def fieldinit(sys: FieldSystem, fields: Dict[int, np.ndarray]):
    """fieldinit!(sys, ::Dict) — src/fileio.jl:25-54 (same-shape case)."""
    for mid, arr in fields.items():
        if mid in sys.monomers:
            arr = np.asarray(arr, dtype=np.float64)
            if arr.shape != sys.shape:
                raise ValueError(f"Input field dimensions {arr.shape} does not match system grid {sys.shape}.")
            sys.fields[mid] = arr.copy()
    sys.residuals_update()


def loadfields(path: str) -> dict:
    """loadfields — src/fileio.jl:99-132.  Nested [z][y][x] lists become (Nz, Ny, Nx)."""
    import json
    with open(path) as fh:
        raw = json.load(fh)
    grid = tuple(int(g) for g in raw["grid"])
    mids = [int(m) for m in raw["mids"]]
    fields = {}
    for mid in mids:
        vecs = raw["fields"][str(mid)]
        fields[mid] = np.array(vecs, dtype=np.float64).reshape(grid[2], grid[1], grid[0])
    return {"dim": int(raw["dim"]), "grid": grid, "mids": mids, "crystal": raw["crystal"],
            "cell_params": [float(p) for p in raw["cell_params"]],
            "field_type": raw["field_type"], "fields": fields}
