"""Python mirror of PolyFields.jl's public API, computing on the GB300 through the C ABI.

Names follow the reference's exports (src/PolyFields.jl:29-45) with the Julia ``!`` dropped:
``add_species!`` is ``add_species``, ``scft!`` is ``scft``, ``fieldinit!`` is ``fieldinit``.
Objects keep the reference's fields (``Multiblock.Nref``, ``.f_block``, ``.begin_block``,
``FieldSystem.fields[mid]`` ...), so scripts written against the reference read the same.
Errors are raised where the reference raises them, with its messages.
"""
from __future__ import annotations

import ctypes
import json
import os
import warnings
import math
from dataclasses import dataclass, field as dc_field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib as L
from . import julia_random

Canonical = "Canonical"
Grand = "Grand"

FP64 = "fp64"
FP32 = "fp32"
_PREC = {FP64: L.PF_FP64, FP32: L.PF_FP32}


# =============================================================================
# Monomers, cells, species, interactions (host descriptors)
# =============================================================================
@dataclass(frozen=True)
class Monomer:
    """src/system/monomer.jl:7-25."""
    id: int
    vol: float = 1.0
    charge: float = 0.0


class UnitCell:
    """UnitCell(dim, crystal, params...) — src/system/cell.jl:31-54.  The basis matrices are
    computed by the engine once the cell is attached to a system."""

    def __init__(self, dim: int, crystal: str, *params):
        if len(params) == 1 and isinstance(params[0], (list, tuple, np.ndarray)):
            params = tuple(params[0])
        self.dim = int(dim)
        self.crystal = str(crystal).lstrip(":")
        self._params = np.array(params, dtype=np.float64)
        self._sys = None

    @property
    def params(self) -> np.ndarray:
        if self._sys is not None:
            out = np.zeros(len(self._params))
            vol = ctypes.c_double()
            L.check(L.load().pf_get_cell(self._sys._h, L.dptr(out), len(out), ctypes.byref(vol)), self._sys._h)
            return out
        return self._params.copy()

    @property
    def volume(self) -> float:
        if self._sys is None:
            raise RuntimeError("the cell volume is computed once the cell belongs to a FieldSystem")
        vol = ctypes.c_double()
        L.check(L.load().pf_get_cell(self._sys._h, None, 0, ctypes.byref(vol)), self._sys._h)
        return vol.value

    @property
    def nparams(self) -> int:
        return len(self._params)


def chain_grid(N_block: Sequence[float], Ns: int):
    """src/species/base.jl:27-56."""
    N = float(sum(N_block))
    ds = N / Ns
    begin_block = [1]
    ds_block = []
    bgn = 1
    for nb in N_block:
        Ns_half = int(math.floor(nb / ds / 2.0 + 0.5))
        if Ns_half == 0:
            Ns_half = 1
            ds_block.append(nb / 2.0)
        else:
            ds_block.append(nb / Ns_half / 2.0)
        bgn += Ns_half * 2
        begin_block.append(bgn)
    return N, begin_block, ds_block


class Multiblock:
    """src/species/multiblock.jl:5-60."""

    def __init__(self, mon_block: Sequence[Monomer], N_block: Sequence[int], b_block: Sequence[float],
                 Ns: int = 100):
        assert len(mon_block) == len(N_block) == len(b_block)
        self.monomers = sorted(set(mon_block), key=lambda m: m.id)
        self.mids = [m.id for m in self.monomers]
        self.mid_block = [m.id for m in mon_block]
        self.mid_map: Dict[int, List[int]] = {}
        for i, mid in enumerate(self.mid_block):
            self.mid_map.setdefault(mid, []).append(i)
        self.N = int(sum(N_block))
        self.N_block = [int(n) for n in N_block]
        self.Nref_block = [mon_block[i].vol * N_block[i] for i in range(len(mon_block))]
        self.Nref, self.begin_block, self.ds_block = chain_grid(self.Nref_block, Ns)
        self.f_block = [v / self.Nref for v in self.Nref_block]
        self.b_block = [float(b) for b in b_block]
        self.Ns = self.begin_block[-1] - 1
        self._sys = None
        self._isp = -1

    @property
    def nblocks(self) -> int:
        return len(self.N_block)

    def hasmonomer(self, mid: int) -> bool:
        return mid in self.mids

    def monomer_fraction(self, mid: int) -> float:
        if not self.hasmonomer(mid):
            return 0.0
        return sum(self.f_block[i] for i in self.mid_map[mid])

    @property
    def Q(self) -> float:
        return self._sys._species_q(self._isp)

    def propagator(self, s: int, conjugate: bool = False) -> np.ndarray:
        """chain.q[s+1] / chain.qc[s+1] of the reference (s 0-based) from the last density solve."""
        return self._sys._propagator(self._isp, conjugate, s)


def Homopolymer(mon: Monomer, N: int, b: float, Ns: int = 100) -> Multiblock:
    """multiblock.jl:62-64."""
    return Multiblock([mon], [N], [b], Ns)


def Diblock(amon: Monomer, bmon: Monomer, N: int, f: float, b1: float, b2: float, Ns: int = 100) -> Multiblock:
    """multiblock.jl:66-72."""
    N_block = [int(f * N), int((1 - f) * N)]
    if sum(N_block) != N:
        raise ValueError(f"Non-integer block lengths for N = {N}, f = {f}.")
    return Multiblock([amon, bmon], N_block, [b1, b2], Ns)


class Point:
    """src/species/point.jl:9-22."""

    def __init__(self, mon: Monomer):
        self.mids = [mon.id]
        self.Nref = mon.vol
        self._sys = None
        self._isp = -1

    def hasmonomer(self, mid: int) -> bool:
        return mid in self.mids

    def monomer_fraction(self, mid: int) -> float:
        return 1.0 if self.hasmonomer(mid) else 0.0

    @property
    def Q(self) -> float:
        return self._sys._species_q(self._isp)


class FloryInteraction:
    """src/interactions/flory.jl:9-49."""

    def __init__(self):
        self.mids = set()
        self.chis: Dict[tuple, float] = {}

    def set_interaction(self, alpha, beta, chi: float):
        alpha = alpha.id if isinstance(alpha, Monomer) else int(alpha)
        beta = beta.id if isinstance(beta, Monomer) else int(beta)
        assert alpha != beta
        pair = (alpha, beta) if alpha <= beta else (beta, alpha)
        self.mids.update((alpha, beta))
        self.chis[pair] = float(chi)


class EdwardsInteraction:
    """src/interactions/edwards.jl:9-87: excluded volume (u/2) sum_i (rho_i / v_i)^2."""

    def __init__(self):
        self.mids = set()
        self.uvals: Dict[int, float] = {}

    def set_interaction(self, mid, u: float):
        mid = mid.id if isinstance(mid, Monomer) else int(mid)
        self.mids.add(mid)
        self.uvals[mid] = float(u)


def set_interaction(itx: FloryInteraction, alpha, beta, chi: float):
    itx.set_interaction(alpha, beta, chi)


# =============================================================================
# FieldSystem
# =============================================================================
class _GridView:
    """Dict-like view of one family of device grids, keyed by monomer id."""

    def __init__(self, sys: "FieldSystem", kind: int):
        self._sys, self._kind = sys, kind

    def __getitem__(self, mid: int) -> np.ndarray:
        out = np.empty(self._sys.shape)
        L.check(L.load().pf_get_grid(self._sys._h, self._kind, int(mid), L.dptr(out)), self._sys._h)
        return out

    def __setitem__(self, mid: int, arr) -> None:
        if self._kind != L.PF_FIELD:
            raise TypeError("only fields can be assigned")
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.shape != self._sys.shape:
            raise ValueError(f"Input field dimensions {a.shape} does not match system grid {self._sys.shape}.")
        L.check(L.load().pf_set_field(self._sys._h, int(mid), L.dptr(a)), self._sys._h)

    def keys(self):
        return list(self._sys.monomers.keys())

    def __iter__(self):
        return iter(self.keys())

    def items(self):
        return [(k, self[k]) for k in self.keys()]

    def values(self):
        return [self[k] for k in self.keys()]


class FieldSystem:
    """FieldSystem(dims, cell; monomers, ensemble) — src/system/system.jl:51-76.

    ``precision`` selects the propagator arithmetic: "fp64" (the reference's) or "fp32"
    (densities, residuals, reductions, Anderson and stress sums stay float64)."""

    def __init__(self, dims, cell: UnitCell, monomers: Sequence[Monomer] = (), ensemble: str = Canonical,
                 precision: str = FP64, mde: str = "RK2"):
        if ensemble not in (Canonical, Grand):
            raise ValueError(f"unknown ensemble {ensemble}")
        mde = str(mde).lstrip(":")
        if mde not in ("RK2", "RQM4"):
            raise ValueError(f"Invalid propagator method `{mde}` for PseudoSpectralSolver.")
        dims = tuple(int(d) for d in dims)
        if tuple(sorted(dims, reverse=True)) != dims:
            raise AssertionError("dims must be given in descending order (src/system/system.jl:58)")
        lib = L.load()
        h = ctypes.c_void_p()
        st = lib.pf_system_create(ctypes.byref(h), dims[0], dims[1], dims[2], _PREC[precision])
        if st != L.PF_OK:
            raise L.PolyFieldsError(st, f"pf_system_create{dims}: {lib.pf_status_string(st).decode()}")
        self._h = h
        if ensemble == Grand:
            L.check(lib.pf_set_ensemble(h, 1), h)
        if mde == "RQM4":
            L.check(lib.pf_set_mde(h, 1), h)
        self.mde = mde
        self.dims = dims
        self.shape = (dims[2], dims[1], dims[0])
        self.ensemble = ensemble
        self.monomers: Dict[int, Monomer] = {}
        self.species: list = []
        self.phi_species: List[float] = []
        self.interactions: list = []
        self.cell = None
        self.add_cell(cell)
        for m in monomers:
            self.add_monomer(m)
        self.fields = _GridView(self, L.PF_FIELD)
        self.density = _GridView(self, L.PF_DENSITY)
        self.residuals = _GridView(self, L.PF_RESIDUAL)
        self.potentials = _GridView(self, L.PF_POTENTIAL)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                L.load().pf_system_destroy(h)
            except Exception:
                pass
            self._h = None

    # -- composition
    @property
    def ngrid(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    @property
    def precision(self) -> str:
        p = ctypes.c_int()
        L.check(L.load().pf_get_precision(self._h, ctypes.byref(p)), self._h)
        return FP64 if p.value == L.PF_FP64 else FP32

    @precision.setter
    def precision(self, value: str) -> None:
        L.check(L.load().pf_set_precision(self._h, _PREC[value]), self._h)

    def set_signed_k(self, on: bool = True) -> None:
        """Signed y/z frequencies in |k|^2 instead of the reference's |j| fold (cell.jl:276-277,
        306-307, which changes |k|^2 in non-orthogonal cells); off by default, as in the
        reference."""
        L.check(L.load().pf_set_signed_k(self._h, 1 if on else 0), self._h)

    def add_cell(self, cell: UnitCell) -> None:
        p = np.ascontiguousarray(cell._params, dtype=np.float64)
        L.check(L.load().pf_set_cell(self._h, cell.dim, cell.crystal.encode(), L.dptr(p), len(p)), self._h)
        cell._sys = self
        self.cell = cell

    def add_monomer(self, mon: Monomer) -> None:
        L.check(L.load().pf_add_monomer(self._h, mon.id, mon.vol, mon.charge), self._h)
        self.monomers[mon.id] = mon

    def add_species(self, species, val: float) -> None:
        lib = L.load()
        if isinstance(species, Multiblock):
            mids = np.array(species.mid_block, dtype=np.int32)
            Nb = np.array(species.N_block, dtype=np.int32)
            bb = np.array(species.b_block, dtype=np.float64)
            for mid in species.mid_block:
                if mid in self.monomers and self.monomers[mid] not in species.monomers:
                    raise ValueError(f"monomer {mid} of the species differs from the system's")
            L.check(lib.pf_add_multiblock(self._h, len(mids), L.iptr(mids), L.iptr(Nb), L.dptr(bb),
                                          species.Ns, float(val)), self._h)
        elif isinstance(species, Point):
            L.check(lib.pf_add_point(self._h, species.mids[0], float(val)), self._h)
        else:
            raise TypeError(f"unsupported species {type(species).__name__}")
        species._sys = self
        species._isp = len(self.species)
        self.species.append(species)
        self.phi_species.append(float(val))

    def add_interaction(self, itx) -> None:
        if isinstance(itx, FloryInteraction):
            for (a, b), chi in itx.chis.items():
                L.check(L.load().pf_set_flory(self._h, a, b, chi), self._h)
        elif isinstance(itx, EdwardsInteraction):
            for mid, u in itx.uvals.items():
                L.check(L.load().pf_set_edwards(self._h, mid, u), self._h)
        else:
            raise TypeError("the GPU engine implements FloryInteraction and EdwardsInteraction")
        self.interactions.append(itx)

    # -- hot path (system.jl)
    def validate(self) -> None:
        L.check(L.load().pf_validate(self._h), self._h)

    def density_update(self) -> None:
        L.check(L.load().pf_density(self._h), self._h)

    def residuals_update(self) -> None:
        L.check(L.load().pf_residuals(self._h), self._h)

    def free_energy(self) -> float:
        v = ctypes.c_double()
        L.check(L.load().pf_free_energy(self._h, ctypes.byref(v)), self._h)
        return v.value

    def free_energy_bulk(self) -> float:
        v = ctypes.c_double()
        L.check(L.load().pf_free_energy_bulk(self._h, ctypes.byref(v)), self._h)
        return v.value

    def field_error(self) -> float:
        v = ctypes.c_double()
        L.check(L.load().pf_field_error(self._h, ctypes.byref(v)), self._h)
        return v.value

    def scfstress(self) -> np.ndarray:
        out = np.zeros(self.cell.nparams)
        L.check(L.load().pf_scfstress(self._h, L.dptr(out), len(out)), self._h)
        return out

    def _species_q(self, isp: int) -> float:
        v = ctypes.c_double()
        L.check(L.load().pf_species_q(self._h, isp, ctypes.byref(v)), self._h)
        return v.value

    def _propagator(self, isp: int, conjugate: bool, s: int) -> np.ndarray:
        out = np.empty(self.shape)
        L.check(L.load().pf_get_propagator(self._h, isp, 1 if conjugate else 0, s, L.dptr(out)), self._h)
        return out

    def set_adjoint_checkpoints(self, every: int) -> None:
        """Pullback reads the propagators only every ``every`` contour steps and recomputes the
        steps in between (0: read all stored steps)."""
        L.check(L.load().pf_set_adjoint_checkpoints(self._h, int(every)), self._h)

    def density_pullback(self, rho_bar: Dict[int, np.ndarray]) -> Dict:
        """Pullback of density!(sys) for a loss L with dL/drho_m = rho_bar[m] (monomers not
        listed: zero).  Recomputes the density at the current fields and cell, then returns
        {"w": {mid: dL/dw_mid}, "cell": dL/dtheta, "Nref_block": [per species, dL/dNref_b of
        each block (empty for point species)], "chi": {pair: 0.0}}."""
        lib = L.load()
        for mid in self.monomers:
            arr = rho_bar.get(mid)
            if arr is None:
                L.check(lib.pf_set_density_cotangent(self._h, mid, None), self._h)
            else:
                a = np.ascontiguousarray(arr, dtype=np.float64)
                if a.shape != self.shape:
                    raise ValueError(f"cotangent of monomer {mid} has shape {a.shape}, expected {self.shape}")
                L.check(lib.pf_set_density_cotangent(self._h, mid, L.dptr(a)), self._h)
        npr = len(self.cell.params)
        nblk = [len(sp.N_block) if isinstance(sp, Multiblock) else 0 for sp in self.species]
        cell_bar = np.zeros(max(1, npr))
        nref = np.zeros(max(1, sum(nblk)))
        L.check(lib.pf_density_pullback(self._h, L.dptr(cell_bar), npr, L.dptr(nref), sum(nblk)), self._h)
        out = {"w": {}, "cell": cell_bar[:npr].copy(), "Nref_block": [], "chi": {}}
        for mid in self.monomers:
            g = np.empty(self.shape)
            L.check(lib.pf_get_grid(self._h, L.PF_FIELD_COTANGENT, mid, L.dptr(g)), self._h)
            out["w"][mid] = g
        k = 0
        for n in nblk:
            out["Nref_block"].append(list(nref[k:k + n]))
            k += n
        for itx in self.interactions:
            for pair in getattr(itx, "chis", {}):
                out["chi"][pair] = 0.0
        return out

    def free_energy_pullback(self) -> Dict:
        """Gradient of free_energy (src/system/system.jl:402-433) at the current fields and cell:
        {"fhelm": value, "w": {mid: dF/dw_mid}, "cell": dF/dtheta, "Nref_block": [per species,
        dF/dNref_b of each block (empty for point species)], "chi": {(a, b): dF/dchi_ab},
        "u": {mid: dF/du_mid}}.  Solves density! first; replaces the density cotangent."""
        lib = L.load()
        npr = len(self.cell.params)
        nblk = [len(sp.N_block) if isinstance(sp, Multiblock) else 0 for sp in self.species]
        pairs = sorted({pair for itx in self.interactions for pair in getattr(itx, "chis", {})})
        umids = sorted({m for itx in self.interactions for m in getattr(itx, "uvals", {})})
        cell_bar = np.zeros(max(1, npr))
        nref = np.zeros(max(1, sum(nblk)))
        chi = np.zeros(max(1, len(pairs)))
        ub = np.zeros(max(1, len(umids)))
        f = ctypes.c_double()
        L.check(lib.pf_free_energy_pullback(self._h, L.dptr(cell_bar), npr, L.dptr(nref), sum(nblk), L.dptr(chi),
                                            len(pairs), L.dptr(ub), len(umids), ctypes.byref(f)), self._h)
        out = {"fhelm": f.value, "w": {}, "cell": cell_bar[:npr].copy(), "Nref_block": [],
               "chi": {pair: float(chi[i]) for i, pair in enumerate(pairs)},
               "u": {m: float(ub[i]) for i, m in enumerate(umids)}}
        for mid in self.monomers:
            g = np.empty(self.shape)
            L.check(lib.pf_get_grid(self._h, L.PF_FIELD_COTANGENT, mid, L.dptr(g)), self._h)
            out["w"][mid] = g
        k = 0
        for n in nblk:
            out["Nref_block"].append(list(nref[k:k + n]))
            k += n
        return out

    def set_wait_limit(self, seconds: float) -> None:
        """Time limit of the 3D pencil passes' bounded waits for their TMA copies (default 1 s).
        A wait that runs out invalidates the solve: the next call that reads results raises
        PolyFieldsError with status PF_ETIMEOUT, and the handle stays usable.  0 makes every
        such wait give up at once (exercises the timeout path in tests)."""
        L.check(L.load().pf_set_wait_limit(self._h, float(seconds)), self._h)

    def pencil_schedule(self):
        """(stages, rounds, tuned) of the 3D pencil pass for this grid and precision: the
        autotuner's choice once a density has been solved on this grid (tuned True)."""
        a, b, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.check(L.load().pf_get_pencil_schedule(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(t)),
                self._h)
        return a.value, b.value, bool(t.value)

    def set_timing(self, enable: bool) -> None:
        L.check(L.load().pf_set_timing(self._h, 1 if enable else 0), self._h)

    def last_timing(self):
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        L.check(L.load().pf_last_timing(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)), self._h)
        return a.value, b.value, n.value

    def synchronize(self) -> None:
        L.check(L.load().pf_synchronize(self._h), self._h)


def add_monomer(sys: FieldSystem, mon: Monomer) -> None:
    """add_monomer!(sys, mon) (system.jl:113-128)."""
    sys.add_monomer(mon)


def add_cell(sys: FieldSystem, cell: UnitCell) -> None:
    """add_cell!(sys, cell) (system.jl:102-106)."""
    sys.add_cell(cell)


def add_species(sys: FieldSystem, species, val: float) -> None:
    sys.add_species(species, val)


def monomer_fraction(species, mid: int) -> float:
    """monomer_fraction(species, mid) (multiblock.jl:93-102, point.jl)."""
    return species.monomer_fraction(int(mid))


def uniform_fields(sys: FieldSystem) -> None:
    """uniform_fields!(sys) (system.jl:348-357): every field becomes the potential of the current
    densities, mean-subtracted in the canonical ensemble."""
    rho = {mid: sys.density[mid] for mid in sys.monomers}
    for mid, pot in _potentials_from(sys, rho).items():
        sys.fields[mid] = pot - np.mean(pot) if sys.ensemble == Canonical else pot


def add_interaction(sys: FieldSystem, itx) -> None:
    sys.add_interaction(itx)


def validate(sys: FieldSystem) -> None:
    sys.validate()


def density(sys: FieldSystem) -> None:
    """density!(sys)."""
    sys.density_update()


def residuals(sys: FieldSystem) -> None:
    """residuals!(sys)."""
    sys.residuals_update()


def free_energy(sys: FieldSystem) -> float:
    return sys.free_energy()


def free_energy_bulk(sys: FieldSystem) -> float:
    return sys.free_energy_bulk()


def field_error(sys: FieldSystem) -> float:
    return sys.field_error()


def scfstress(sys: FieldSystem) -> np.ndarray:
    return sys.scfstress()


# =============================================================================
# Updaters and driver
# =============================================================================
class AndersonUpdater:
    """AndersonUpdater(; nhist = 50, iter_euler = 1, lam_euler = 0.01) — anderson.jl:36-47.
    The history lives on the device of the system it is set up with.  The engine keeps one
    Anderson history per system: once a second AndersonUpdater is set up on a system, the
    first one raises RuntimeError instead of stepping with the second one's history."""

    def __init__(self, nhist: int = 50, iter_euler: int = 1, lam_euler: float = 0.01):
        self.nhist = int(nhist)
        self.iter_euler = max(1, int(iter_euler))
        self.lam_euler = float(lam_euler)
        self.system: Optional[FieldSystem] = None

    def _owns(self, sys: FieldSystem) -> None:
        if getattr(sys, "_anderson", None) is not self:
            raise RuntimeError("another AndersonUpdater was set up on this system since; the GPU engine keeps "
                               "one Anderson history per system")

    def _bind(self, sys: FieldSystem) -> None:
        """Create the updater's history on sys (once per system) and make it the current one."""
        if self.system is not sys:
            L.check(L.load().pf_anderson_create(sys._h, self.nhist, self.iter_euler, self.lam_euler), sys._h)
            self.system = sys
            sys._anderson = self
        else:
            self._owns(sys)
            L.check(L.load().pf_updater_select(sys._h, -1), sys._h)

    def setup(self, sys: FieldSystem) -> None:
        """setup!(updater, sys) — anderson.jl:54-92."""
        self._bind(sys)
        L.check(L.load().pf_anderson_setup(sys._h), sys._h)

    def step(self) -> None:
        """step!(updater) — anderson.jl:98-228."""
        if self.system is None:
            raise RuntimeError("AndersonUpdater is not set up")
        self._owns(self.system)
        L.check(L.load().pf_anderson_step(self.system._h), self.system._h)


class _SimpleUpdater:
    """State of an Euler or Momentum updater on the device of its system.  Each updater object
    owns its own state there (created on first use with a system), so several updaters can be
    set up on one system and stepped in turn, as test/test_updaters.jl:16-30 does."""

    system: Optional[FieldSystem] = None
    _id: int = -1

    def _create(self, sys: FieldSystem) -> None:
        raise NotImplementedError

    def _bind(self, sys: FieldSystem) -> None:
        lib = L.load()
        if self.system is not sys:
            self._create(sys)
            uid = ctypes.c_int()
            L.check(lib.pf_updater_current(sys._h, ctypes.byref(uid)), sys._h)
            self.system, self._id = sys, uid.value
        else:
            L.check(lib.pf_updater_select(sys._h, self._id), sys._h)

    def setup(self, sys: FieldSystem) -> None:
        """setup!(updater, sys) — euler.jl:31-35, momentum.jl:49-61."""
        self._bind(sys)
        L.check(L.load().pf_updater_setup(sys._h), sys._h)

    def step(self) -> None:
        """step!(updater) — euler.jl:37-65, momentum.jl:63-165."""
        if self.system is None:
            raise RuntimeError(f"{type(self).__name__} is not set up")
        self._bind(self.system)
        L.check(L.load().pf_updater_step(self.system._h), self.system._h)


class EulerUpdater(_SimpleUpdater):
    """EulerUpdater(; method = :PECE, lam = 0.05) — euler.jl:9-29 (predictor-corrector Euler)."""

    _METHODS = {"PEC": 0, "PECE": 1}

    def __init__(self, method: str = "PECE", lam: float = 0.05):
        method = str(method).lstrip(":")
        if method not in self._METHODS:
            raise ValueError("Invalid `method` parameter for EulerUpdater. Options include: (:PEC, :PECE)")
        self.method, self.lam = method, float(lam)
        self.system: Optional[FieldSystem] = None

    def _create(self, sys: FieldSystem) -> None:
        L.check(L.load().pf_euler_create(sys._h, self._METHODS[self.method], self.lam), sys._h)


class MomentumUpdater(_SimpleUpdater):
    """MomentumUpdater(; method = :MOM, lam = 0.01, gamma = 0.9, beta1 = 0.9, beta2 = 0.999)
    — momentum.jl:19-47 (MOM, RMS, ADAM, NAG)."""

    _METHODS = {"MOM": 0, "RMS": 1, "ADAM": 2, "NAG": 3}

    def __init__(self, method: str = "MOM", lam: float = 0.01, gamma: float = 0.9, beta1: float = 0.9,
                 beta2: float = 0.999):
        assert 0.0 < gamma < 1.0 and 0.0 < beta1 < 1.0 and 0.0 < beta2 < 1.0
        method = str(method).lstrip(":")
        if method not in self._METHODS:
            raise ValueError("Invalid `method` parameter for MomentumUpdater. Options include: (:MOM, :RMS, :ADAM, :NAG)")
        self.method, self.lam = method, float(lam)
        self.gamma, self.beta1, self.beta2 = float(gamma), float(beta1), float(beta2)
        self.system: Optional[FieldSystem] = None

    def _create(self, sys: FieldSystem) -> None:
        L.check(L.load().pf_momentum_create(sys._h, self._METHODS[self.method], self.lam, self.gamma, self.beta1,
                                            self.beta2), sys._h)


class DomainUpdater:
    """DomainUpdater(; nper = 10, nskip = 200, lam = 0.1, pmax = 1.0, rlxn = 0.5) — domain.jl:20-24."""

    def __init__(self, nper: int = 10, nskip: int = 200, lam: float = 0.1, pmax: float = 1.0, rlxn: float = 0.5):
        self.nper, self.nskip = int(nper), int(nskip)
        self.lam, self.pmax, self.rlxn = float(lam), float(pmax), float(rlxn)
        self.system: Optional[FieldSystem] = None

    def _bind(self, sys: FieldSystem) -> None:
        L.check(L.load().pf_domain_create(sys._h, self.nper, self.nskip, self.lam, self.pmax, self.rlxn), sys._h)
        self.system = sys

    def setup(self, sys: FieldSystem) -> None:
        self._bind(sys)
        L.check(L.load().pf_domain_setup(sys._h), sys._h)

    def step(self, nsteps: int = 1, tol: float = 1e-5) -> None:
        L.check(L.load().pf_domain_step(self.system._h, int(nsteps)), self.system._h)

    def stress_error(self) -> float:
        v = ctypes.c_double()
        L.check(L.load().pf_domain_stress_error(self.system._h, ctypes.byref(v)), self.system._h)
        return v.value


def updater_with_system(cls, sys: FieldSystem, **kwargs):
    """src/updaters/base.jl:16-20."""
    u = cls(**kwargs)
    u.setup(sys)
    return u


def setup(updater, sys: FieldSystem) -> None:
    updater.setup(sys)


def step(updater, **kwargs) -> None:
    updater.step(**kwargs)


@dataclass
class SCFTOptions:
    """src/simulate.jl:12-19, plus ``mixed_switch_ferr``: with an fp32 system, iterate in fp32
    until ferr < mixed_switch_ferr (or until 200 fp32 iterations bring no 1% improvement),
    then continue in fp64 (0 disables the switch).  ``polish`` selects the fp64 phase:
    "newton" (Newton-Krylov steps: one fp64 residual each, the linear solve by GMRES over
    fp32 finite-difference Jacobian products; runs without a DomainUpdater, falls back to the
    updater's fp64 steps if a Newton step stalls), "updater" (fp64 steps of the field
    updater), or "auto" (Newton-Krylov on 3D grids, updater steps on 1D/2D grids)."""
    nsteps: int = 100
    nsout: int = 0
    nsave: int = 0
    ftol: float = 1e-5
    stol: float = 1e-4
    savepath: str = ""
    mixed_switch_ferr: float = 0.0
    polish: str = "auto"


@dataclass
class SCFTResults:
    """src/simulate.jl:26-33 (+ the step at which the precision switched, -1 if never)."""
    time: float
    nsteps: int
    converged: bool
    ferr: float
    serr: float
    fhelm: float
    switch_step: int = -1
    polish_fp64_solves: int = 0
    polish_fp32_solves: int = 0


_POLISH = {"auto": 0, "updater": 1, "newton": 2}


def _options(opts: "SCFTOptions"):
    if opts.polish not in _POLISH:
        raise ValueError(f"polish must be one of {sorted(_POLISH)}")
    return L.ScftOptions(opts.nsteps, opts.nsout, opts.nsave, _POLISH[opts.polish], opts.ftol, opts.stol,
                         opts.mixed_switch_ferr)


def _results(r) -> "SCFTResults":
    return SCFTResults(r.time, r.nsteps, bool(r.converged), r.ferr, r.serr, r.fhelm, r.switch_step,
                       r.polish_fp64_solves, r.polish_fp32_solves)


def scft(sys: FieldSystem, updater: AndersonUpdater, domain: Optional[DomainUpdater] = None,
         opts: Optional[SCFTOptions] = None) -> SCFTResults:
    """scft!(sys, updater; domain, opts) — src/simulate.jl:60-148."""
    if not isinstance(updater, (AndersonUpdater, EulerUpdater, MomentumUpdater)):
        raise TypeError("the GPU engine implements scft! with the Anderson, Euler and Momentum updaters")
    opts = opts or SCFTOptions()
    updater._bind(sys)
    if domain is not None:
        domain._bind(sys)
    o = _options(opts)
    r = L.ScftResults()
    lib = L.load()
    L.check(lib.pf_set_savepath(sys._h, (opts.savepath or "").encode()), sys._h)
    L.check(lib.pf_scft(sys._h, ctypes.byref(o), 1 if domain is not None else 0, ctypes.byref(r)), sys._h)
    return _results(r)


def scft_batch(systems: Sequence[FieldSystem], updaters: Sequence[AndersonUpdater],
               domains: Optional[Sequence[Optional[DomainUpdater]]] = None, opts: Optional[SCFTOptions] = None,
               nthreads: int = 0, raise_on_error: bool = True):
    """scft!(sys_i, updater_i; domain_i, opts) for many independent systems at once (a sweep).

    Every system runs on its own CUDA stream; ``nthreads`` host threads (0: up to 32) drive
    them, longest solves first, so the GPU works on up to ``nthreads`` solves concurrently.
    Returns one SCFTResults per system, or, with ``raise_on_error=False``, (results, statuses)
    where statuses[i] is the pf status of system i (0 = ok)."""
    n = len(systems)
    if len(updaters) != n:
        raise ValueError("one AndersonUpdater per system")
    domains = list(domains) if domains is not None else [None] * n
    if len(domains) != n:
        raise ValueError("one DomainUpdater (or None) per system")
    use_domain = domains[0] is not None
    if any((d is not None) != use_domain for d in domains):
        raise ValueError("either every system or none has a DomainUpdater")
    opts = opts or SCFTOptions()
    for sys, u, d in zip(systems, updaters, domains):
        if not isinstance(u, AndersonUpdater):
            raise TypeError("the GPU engine implements scft! with the AndersonUpdater")
        u._bind(sys)
        if d is not None:
            d._bind(sys)
    handles = (L._vp * n)(*[s._h for s in systems])
    o = _options(opts)
    res = (L.ScftResults * n)()
    st = (ctypes.c_int * n)()
    rc = L.load().pf_scft_batch(handles, n, ctypes.byref(o), 1 if use_domain else 0, res, st, int(nthreads))
    out = [_results(r) for r in res]
    if raise_on_error:
        for i in range(n):
            L.check(st[i], systems[i]._h)
        L.check(rc)
        return out
    return out, list(st)


# =============================================================================
# Field initialisation and IO (src/fileio.jl)
# =============================================================================
def _natural_spline_along(a: np.ndarray, axis: int, pos: np.ndarray) -> np.ndarray:
    """Interpolating natural cubic spline (second derivative 0 at both ends) through the samples
    of ``a`` at integer positions 0..n-1 along ``axis``, evaluated at the real positions ``pos``."""
    a = np.moveaxis(np.asarray(a, dtype=np.float64), axis, 0)
    n = a.shape[0]
    flat = a.reshape(n, -1)
    m = np.zeros_like(flat)  # second derivatives at the knots
    if n > 2:
        # (m[i-1] + 4 m[i] + m[i+1]) = 6 (y[i-1] - 2 y[i] + y[i+1]),  m[0] = m[n-1] = 0 (Thomas)
        rhs = 6.0 * (flat[:-2] - 2.0 * flat[1:-1] + flat[2:])
        k = n - 2
        c = np.zeros(k)
        d = np.zeros_like(rhs)
        c[0] = 1.0 / 4.0
        d[0] = rhs[0] / 4.0
        for i in range(1, k):
            den = 4.0 - c[i - 1]
            c[i] = 1.0 / den
            d[i] = (rhs[i] - d[i - 1]) / den
        x = np.zeros_like(rhs)
        x[-1] = d[-1]
        for i in range(k - 2, -1, -1):
            x[i] = d[i] - c[i] * x[i + 1]
        m[1:-1] = x
    j = np.clip(np.floor(pos).astype(int), 0, max(n - 2, 0))
    t = (pos - j)[:, None]
    if n == 1:
        out = np.repeat(flat[:1], len(pos), axis=0)
    else:
        y0, y1, m0, m1 = flat[j], flat[j + 1], m[j], m[j + 1]
        out = (1 - t) * y0 + t * y1 + ((1 - t) ** 3 - (1 - t)) * m0 / 6.0 + (t ** 3 - t) * m1 / 6.0
    return np.moveaxis(out.reshape((len(pos),) + a.shape[1:]), 0, axis)


def interpolate_grid(grid: np.ndarray, dims) -> np.ndarray:
    """interpolate_grid(grid, outshape) (src/utils.jl:64-109): a field or density grid of shape
    (Nz, Ny, Nx) resampled to ``dims`` = (Nx', Ny', Nz') by the cubic B-spline with linear ("Line",
    zero second derivative) boundaries that the reference builds with Interpolations.jl
    (BSpline(Cubic(Line(OnGrid())))): on the grid points that is the interpolating natural cubic
    spline, applied axis by axis (the tensor-product spline factorises).  As in the reference the
    output points run from the first to the last input point (range(1, n_in; length = n_out)); an
    axis of length 1 in the input is copied along the output axis, an output axis of length 1
    takes the first input point."""
    grid = np.asarray(grid, dtype=np.float64)
    if grid.ndim != 3:
        raise ValueError("grid must be a 3-D array of shape (Nz, Ny, Nx)")
    out_shape = (int(dims[2]), int(dims[1]), int(dims[0]))
    in_single = tuple(i for i in range(3) if grid.shape[i] == 1)
    out_single = tuple(i for i in range(3) if out_shape[i] == 1)
    if in_single != out_single:
        warnings.warn("Interpolating to different dimensions -- output array may be inaccurate.")
    a = grid
    for axis in range(3):
        nin, nout = a.shape[axis], out_shape[axis]
        if nin == nout:
            continue
        if nin == 1:
            a = np.repeat(a, nout, axis=axis)
        elif nout == 1:
            a = np.take(a, [0], axis=axis)
        else:
            a = _natural_spline_along(a, axis, np.linspace(0.0, nin - 1.0, nout))
    return np.ascontiguousarray(a)


def _potentials_from(sys: FieldSystem, rho: Dict[int, np.ndarray]) -> Dict[int, np.ndarray]:
    """potentials!(sys) (system.jl:296-310) from given densities: Flory (flory.jl:82-100)
    pot_a += chi_ab rho_b / v_b and Edwards (edwards.jl) pot_a += u_a rho_a / v_a."""
    pots = {mid: np.zeros(sys.shape) for mid in sys.monomers}
    for itx in sys.interactions:
        if isinstance(itx, FloryInteraction):
            for (a, b), chi in itx.chis.items():
                if a in pots and b in rho:
                    pots[a] += chi * (rho[b] / sys.monomers[b].vol)
                if b in pots and a in rho:
                    pots[b] += chi * (rho[a] / sys.monomers[a].vol)
        elif isinstance(itx, EdwardsInteraction):
            for mid, u in itx.uvals.items():
                if mid in pots and mid in rho:
                    pots[mid] += u * (rho[mid] / sys.monomers[mid].vol)
    return pots


def fieldinit(sys: FieldSystem, fields=None, *, field_type: str = "omega", interpolate: bool = True,
              load_cell: bool = True, seed: int = -1, scale: float = 0.1) -> None:
    """fieldinit!(sys, fields::Dict; field_type, interpolate) (fileio.jl:25-54),
    fieldinit!(sys, path; load_cell, interpolate) (fileio.jl:56-64) when ``fields`` is a path to
    a savefields JSON, or, without ``fields``, fieldinit!(sys; seed, scale) (fileio.jl:14-23):
    the reference's seeded stream (Julia's MersenneTwister randn in its Dict order of the
    monomer ids, polyfields.julia_random), so a seed gives the reference's fields; seed < 0
    continues the process-wide stream.

    Grids of another shape are resampled with interpolate_grid (or rejected with
    interpolate=False).  field_type "rho" takes densities: the fields become their potentials,
    mean-subtracted in the canonical ensemble (uniform_fields!, system.jl:348-357)."""
    if isinstance(fields, (str, os.PathLike)):
        data = loadfields(str(fields))
        if load_cell:
            sys.add_cell(UnitCell(data["dim"], data["crystal"], *data["cell_params"]))
        fieldinit(sys, data["fields"], field_type=data["field_type"], interpolate=interpolate)
        return
    if fields is None:
        fields = julia_random.fieldinit_fields(list(sys.monomers), sys.shape, seed, scale)
    ftype = str(field_type).lstrip(":")
    if ftype not in ("omega", "rho"):
        raise ValueError(f"unknown field_type {field_type}")
    given: Dict[int, np.ndarray] = {}
    for mid, arr in fields.items():
        mid = int(mid)
        if mid not in sys.monomers:
            warnings.warn(f"Monomer with ID = {mid} not present in system -- skipping.")
            continue
        arr = np.asarray(arr, dtype=np.float64)
        if arr.shape != sys.shape:
            if not interpolate:
                raise ValueError(f"Input field dimensions {arr.shape[::-1]} does not match system grid {sys.dims}.")
            arr = interpolate_grid(arr, sys.dims)
        given[mid] = arr
    if ftype == "omega":
        for mid, arr in given.items():
            sys.fields[mid] = arr
    else:
        rho = {mid: sys.density[mid] for mid in sys.monomers}
        rho.update(given)
        for mid, pot in _potentials_from(sys, rho).items():
            sys.fields[mid] = pot - np.mean(pot) if sys.ensemble == Canonical else pot
    sys.residuals_update()


def loadfields(path: str) -> dict:
    """loadfields (fileio.jl:99-132): nested [z][y][x] JSON lists -> arrays of shape (Nz, Ny, Nx)."""
    with open(path) as fh:
        raw = json.load(fh)
    grid = tuple(int(g) for g in raw["grid"])
    mids = [int(m) for m in raw["mids"]]
    fields = {m: np.array(raw["fields"][str(m)], dtype=np.float64).reshape(grid[2], grid[1], grid[0]) for m in mids}
    return {"dim": int(raw["dim"]), "grid": grid, "mids": mids, "crystal": raw["crystal"],
            "cell_params": [float(p) for p in raw["cell_params"]], "field_type": raw["field_type"],
            "fields": fields}


def savefields(sys: FieldSystem, path: str, field_type: str = "omega") -> None:
    """savefields (fileio.jl:77-97): the same JSON layout the reference writes."""
    import datetime
    grids = sys.density if field_type == "rho" else sys.fields
    d = {"dim": sum(1 for n in sys.dims if n > 1), "grid": list(sys.dims), "mids": sorted(sys.monomers),
         "date": datetime.datetime.now().strftime("%Y-%m-%d %H:%M:%S"), "crystal": sys.cell.crystal,
         "cell_params": [float(p) for p in sys.cell.params], "field_type": field_type,
         "fields": {str(m): grids[m].tolist() for m in sorted(sys.monomers)}}
    with open(path, "w") as fh:
        json.dump(d, fh, indent=4)
