"""ctypes wrapper of oracle/pf_cpu.cpp, the C++17/OpenMP FP64 CPU restatement of one scft!
iteration (propagators with a project-written FFT, Simpson, residuals, Anderson).

TEST INFRASTRUCTURE: bench.py's CPU baseline and --impl reference arm time it, and the CPU
tests pin it to the NumPy oracle (pf_oracle.py).  The GPU engine never uses it.

    import pf_oracle as O, pf_cpu as C
    o = <an oracle FieldSystem with fields injected>
    c = C.CpuSystem.from_oracle(o, nthreads=0)   # all host threads
    c.residuals(); c.free_energy(); c.anderson_setup(20); c.anderson_step()
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pf_cpu.cpp")
LIB = os.path.join(HERE, "_build", "libpf_cpu.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_SIG = {
    "pfc_create": (_vp, [ctypes.c_int] * 4),
    "pfc_destroy": (None, [_vp]),
    "pfc_threads": (ctypes.c_int, []),
    "pfc_set_ksq": (None, [_vp, _dp]),
    "pfc_add_monomer": (ctypes.c_int, [_vp, ctypes.c_double]),
    "pfc_set_chi": (None, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "pfc_add_multiblock": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp, _ip, ctypes.c_double, ctypes.c_double]),
    "pfc_add_point": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    "pfc_set_field": (None, [_vp, ctypes.c_int, _dp]),
    "pfc_get_grid": (None, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    "pfc_residuals": (None, [_vp]),
    "pfc_field_error": (ctypes.c_double, [_vp]),
    "pfc_free_energy": (ctypes.c_double, [_vp]),
    "pfc_species_q": (ctypes.c_double, [_vp, ctypes.c_int]),
    "pfc_propagate": (None, [_vp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _dp, ctypes.c_int]),
    "pfc_anderson_setup": (None, [_vp, ctypes.c_int]),
    "pfc_anderson_step": (ctypes.c_int, [_vp]),
}
_lib = None


def build(force: bool = False) -> str:
    """g++ -O3 -fopenmp, one translation unit (portable flags: it also builds on the Arm host)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-Wall", SRC, "-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building {LIB} failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        for name, (res, args) in _SIG.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


class CpuSystem:
    """A canonical-ensemble system (Multiblock and Point species, Flory interactions, strict
    incompressibility, RK2) held by the C++ restatement."""

    def __init__(self, dims, ksq, nthreads: int = 0):
        self.lib = load()
        self.dims = tuple(dims)
        self.shape = (dims[2], dims[1], dims[0])
        self.h = self.lib.pfc_create(dims[0], dims[1], dims[2], int(nthreads))
        if not self.h:
            raise RuntimeError("pfc_create failed")
        self._ksq = np.ascontiguousarray(np.broadcast_to(ksq, (dims[2], dims[1], dims[0] // 2 + 1)), dtype=np.float64)
        self.lib.pfc_set_ksq(self.h, _d(self._ksq))
        self.mon_index = {}
        self.nspecies = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.pfc_destroy(self.h)
            self.h = None

    @property
    def threads(self) -> int:
        return self.lib.pfc_threads()

    @classmethod
    def from_oracle(cls, osys, nthreads: int = 0):
        """Copy an oracle FieldSystem's configuration and fields (pf_oracle.FieldSystem)."""
        import pf_oracle as O
        c = cls(osys.dims, osys.cell.ksq, nthreads)
        for mid in sorted(osys.monomers):
            c.mon_index[mid] = c.lib.pfc_add_monomer(c.h, osys.monomers[mid].vol)
        for itx in osys.interactions:
            if not isinstance(itx, O.FloryInteraction):
                raise TypeError("the CPU restatement implements FloryInteraction")
            for (a, b), chi in itx.chis.items():
                c.lib.pfc_set_chi(c.h, c.mon_index[a], c.mon_index[b], chi)
        for isp, sp in enumerate(osys.species):
            phi = osys.phi_species[isp]
            if isinstance(sp, O.Multiblock):
                nb = len(sp.mid_block)
                mon = np.array([c.mon_index[m] for m in sp.mid_block], dtype=np.int32)
                bgn = np.array(sp.begin_block, dtype=np.int32)
                c.lib.pfc_add_multiblock(c.h, nb, mon.ctypes.data_as(_ip), _d(sp.b_block), _d(sp.ds_block),
                                         bgn.ctypes.data_as(_ip), sp.Nref, phi)
            else:
                c.lib.pfc_add_point(c.h, c.mon_index[sp.mids[0]], phi)
            c.nspecies += 1
        for mid, w in osys.fields.items():
            c.set_field(mid, w)
        return c

    def set_field(self, mid, w):
        a = np.ascontiguousarray(w, dtype=np.float64)
        self.lib.pfc_set_field(self.h, self.mon_index[mid], a.ctypes.data_as(_dp))

    def grid(self, kind: int, mid) -> np.ndarray:
        out = np.empty(self.shape)
        self.lib.pfc_get_grid(self.h, kind, self.mon_index[mid], out.ctypes.data_as(_dp))
        return out

    def fields(self, mid):
        return self.grid(0, mid)

    def density(self, mid):
        return self.grid(1, mid)

    def residuals_grid(self, mid):
        return self.grid(2, mid)

    def residuals(self):
        self.lib.pfc_residuals(self.h)

    def field_error(self) -> float:
        return self.lib.pfc_field_error(self.h)

    def free_energy(self) -> float:
        return self.lib.pfc_free_energy(self.h)

    def species_q(self, isp: int) -> float:
        return self.lib.pfc_species_q(self.h, isp)

    def propagate(self, w, vol, b, ds, q0, nsteps):
        out = np.empty(self.shape)
        wa, qa = np.ascontiguousarray(w, np.float64), np.ascontiguousarray(q0, np.float64)
        self.lib.pfc_propagate(self.h, wa.ctypes.data_as(_dp), vol, b, ds, qa.ctypes.data_as(_dp),
                               out.ctypes.data_as(_dp), int(nsteps))
        return out

    def anderson_setup(self, nhist: int):
        self.lib.pfc_anderson_setup(self.h, int(nhist))

    def anderson_step(self):
        st = self.lib.pfc_anderson_step(self.h)
        if st != 0:
            raise RuntimeError(f"Error inverting Umn matrix: SingularException({st})")
