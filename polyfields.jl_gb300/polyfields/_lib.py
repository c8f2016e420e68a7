"""ctypes binding of libpolyfields_gpu.so (C ABI declared in include/polyfields_gpu.h).

The library is the only compute path: when it is missing or no CUDA device is usable the
calls raise; there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpolyfields_gpu.so")

(PF_OK, PF_EARG, PF_ECUDA, PF_ENAN, PF_ESINGULAR, PF_ETIMEOUT, PF_ESTATE, PF_ENOMEM, PF_EUNSUPPORTED,
 PF_ETOOLARGE) = range(10)
PF_FP64, PF_FP32 = 0, 1
PF_FIELD, PF_DENSITY, PF_RESIDUAL, PF_POTENTIAL, PF_FIELD_COTANGENT = range(5)

# Every symbol the header declares, with (restype, argtypes).
_c_int, _c_double, _c_char_p, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_void_p
_dptr = ctypes.POINTER(ctypes.c_double)
_iptr = ctypes.POINTER(ctypes.c_int)


class ScftOptions(ctypes.Structure):
    _fields_ = [("nsteps", _c_int), ("nsout", _c_int), ("nsave", _c_int), ("polish", _c_int),
                ("ftol", _c_double), ("stol", _c_double), ("mixed_switch_ferr", _c_double)]


class ScftResults(ctypes.Structure):
    _fields_ = [("time", _c_double), ("nsteps", _c_int), ("converged", _c_int), ("ferr", _c_double),
                ("serr", _c_double), ("fhelm", _c_double), ("switch_step", _c_int), ("polish_fp64_solves", _c_int),
                ("polish_fp32_solves", _c_int), ("pad0", _c_int)]


SIGNATURES = {
    "pf_version": (_c_int, []),
    "pf_status_string": (_c_char_p, [_c_int]),
    "pf_system_create": (_c_int, [ctypes.POINTER(_vp), _c_int, _c_int, _c_int, _c_int]),
    "pf_system_destroy": (_c_int, [_vp]),
    "pf_last_error": (_c_char_p, [_vp]),
    "pf_set_precision": (_c_int, [_vp, _c_int]),
    "pf_get_precision": (_c_int, [_vp, _iptr]),
    "pf_set_cell": (_c_int, [_vp, _c_int, _c_char_p, _dptr, _c_int]),
    "pf_get_cell": (_c_int, [_vp, _dptr, _c_int, _dptr]),
    "pf_get_basis": (_c_int, [_vp, _dptr, _dptr]),
    "pf_add_monomer": (_c_int, [_vp, _c_int, _c_double, _c_double]),
    "pf_add_multiblock": (_c_int, [_vp, _c_int, _iptr, _iptr, _dptr, _c_int, _c_double]),
    "pf_add_point": (_c_int, [_vp, _c_int, _c_double]),
    "pf_set_flory": (_c_int, [_vp, _c_int, _c_int, _c_double]),
    "pf_species_info": (_c_int, [_vp, _c_int, _iptr, _dptr, _iptr, _dptr, _c_int]),
    "pf_set_field": (_c_int, [_vp, _c_int, _dptr]),
    "pf_get_grid": (_c_int, [_vp, _c_int, _c_int, _dptr]),
    "pf_get_propagator": (_c_int, [_vp, _c_int, _c_int, _c_int, _dptr]),
    "pf_validate": (_c_int, [_vp]),
    "pf_density": (_c_int, [_vp]),
    "pf_residuals": (_c_int, [_vp]),
    "pf_free_energy": (_c_int, [_vp, _dptr]),
    "pf_free_energy_bulk": (_c_int, [_vp, _dptr]),
    "pf_field_error": (_c_int, [_vp, _dptr]),
    "pf_scfstress": (_c_int, [_vp, _dptr, _c_int]),
    "pf_species_q": (_c_int, [_vp, _c_int, _dptr]),
    "pf_anderson_create": (_c_int, [_vp, _c_int, _c_int, _c_double]),
    "pf_anderson_setup": (_c_int, [_vp]),
    "pf_anderson_step": (_c_int, [_vp]),
    "pf_domain_create": (_c_int, [_vp, _c_int, _c_int, _c_double, _c_double, _c_double]),
    "pf_domain_setup": (_c_int, [_vp]),
    "pf_domain_step": (_c_int, [_vp, _c_int]),
    "pf_domain_stress_error": (_c_int, [_vp, _dptr]),
    "pf_scft": (_c_int, [_vp, ctypes.POINTER(ScftOptions), _c_int, ctypes.POINTER(ScftResults)]),
    "pf_set_mde": (_c_int, [_vp, _c_int]),
    "pf_set_savepath": (_c_int, [_vp, ctypes.c_char_p]),
    "pf_set_edwards": (_c_int, [_vp, _c_int, ctypes.c_double]),
    "pf_set_ensemble": (_c_int, [_vp, _c_int]),
    "pf_set_signed_k": (_c_int, [_vp, _c_int]),
    "pf_euler_create": (_c_int, [_vp, _c_int, ctypes.c_double]),
    "pf_momentum_create": (_c_int, [_vp, _c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double]),
    "pf_updater_current": (_c_int, [_vp, ctypes.POINTER(_c_int)]),
    "pf_updater_select": (_c_int, [_vp, _c_int]),
    "pf_updater_setup": (_c_int, [_vp]),
    "pf_updater_step": (_c_int, [_vp]),
    "pf_set_density_cotangent": (_c_int, [_vp, _c_int, _dptr]),
    "pf_set_adjoint_checkpoints": (_c_int, [_vp, _c_int]),
    "pf_density_pullback": (_c_int, [_vp, _dptr, _c_int, _dptr, _c_int]),
    "pf_free_energy_pullback": (_c_int, [_vp, _dptr, _c_int, _dptr, _c_int, _dptr, _c_int, _dptr, _c_int, _dptr]),
    "pf_scft_batch": (_c_int, [ctypes.POINTER(_vp), _c_int, ctypes.POINTER(ScftOptions), _c_int,
                               ctypes.POINTER(ScftResults), ctypes.POINTER(_c_int), _c_int]),
    "pf_propagate": (_c_int, [_vp, _dptr, _c_double, _c_double, _c_double, _dptr, _dptr, _c_int]),
    "pf_propagate_noalloc": (_c_int, [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _c_int, _vp]),
    "pf_propagate_noalloc_status": (_c_int, [_vp]),
    "pf_set_wait_limit": (_c_int, [_vp, _c_double]),
    "pf_get_pencil_schedule": (_c_int, [_vp, _iptr, _iptr, _iptr]),
    "pf_set_timing": (_c_int, [_vp, _c_int]),
    "pf_last_timing": (_c_int, [_vp, _dptr, _dptr, _iptr]),
    "pf_record_event": (_c_int, [_vp, _c_int]),
    "pf_elapsed_ms": (_c_int, [_vp, _c_int, _c_int, _dptr]),
    "pf_launch_count": (ctypes.c_long, []),
    "pf_synchronize": (_c_int, [_vp]),
}

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the shared library (once) and declare every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python polyfields.jl_gb300/build.py` "
                           "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PolyFieldsError(RuntimeError):
    """A failed engine call; ``status`` is the pf_status code."""

    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def check(status: int, handle=None) -> None:
    if status == PF_OK:
        return
    lib = load()
    msg = lib.pf_last_error(handle).decode() if handle else ""
    if not msg:
        msg = lib.pf_status_string(status).decode()
    if status == PF_EARG:
        if msg.startswith("AssertionError"):
            raise AssertionError(msg)
        raise ValueError(msg)
    raise PolyFieldsError(status, msg)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dptr)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_iptr)
