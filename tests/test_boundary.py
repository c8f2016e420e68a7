"""CPU checks of the drop-in boundary: the C-ABI library exports every declared entry point
and the Python mirror's host-side logic matches the reference (no GPU calls)."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import pf_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "polyfields_gpu.h")
LIB = os.path.join(ROOT, "polyfields.jl_gb300", "polyfields", "libpolyfields_gpu.so")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pf_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    if not os.path.exists(LIB):
        subprocess.run([sys.executable, os.path.join(ROOT, "polyfields.jl_gb300", "build.py")], check=True)
    return LIB


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("pf_system_create", "pf_scft", "pf_anderson_step", "pf_domain_step", "pf_scfstress", "pf_propagate"):
        assert n in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(pf_[a-z_0-9]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_binds_every_symbol(lib_path):
    import polyfields._lib as L
    lib = L.load(lib_path)
    assert lib.pf_version() == 100
    assert set(L.SIGNATURES) == set(declared_functions())
    assert lib.pf_status_string(L.PF_ENAN).decode() == "Diverging field updater -- breaking."


def test_python_mirror_chain_grid_matches_oracle():
    import polyfields as pf
    for Nb, Ns in (([50, 50], 100), ([35, 65], 100), ([40, 60], 200), ([50], 200), ([10] * 6, 60), ([3, 97], 100)):
        assert pf.chain_grid(Nb, Ns) == O.chain_grid(Nb, Ns)
    a, b = pf.Monomer(1, 2.0), pf.Monomer(2)
    ch = pf.Diblock(a, b, 100, 0.25, 1.0, 1.0, 200)
    oc = O.Diblock(O.Monomer(1, 2.0), O.Monomer(2), 100, 0.25, 1.0, 1.0, 200)
    assert ch.f_block == oc.f_block and ch.Nref_block == oc.Nref_block and ch.Ns == oc.Ns
    with pytest.raises(ValueError):
        pf.Diblock(a, b, 100, 0.29, 1.0, 1.0, 100)


def test_python_mirror_rejects_unsorted_dims():
    """Quirk Q6 (system.jl:55-58): only descending dims work in the reference, which fails on
    its first size assertion otherwise; the mirror raises the same AssertionError up front."""
    import polyfields as pf
    with pytest.raises(AssertionError):
        pf.FieldSystem((1, 64, 1), pf.UnitCell(1, "lamellar", 10.0))


def test_no_gpu_fails_loudly(lib_path):
    """Without a CUDA device the engine raises instead of falling back to the CPU."""
    import polyfields as pf
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pf.PolyFieldsError):
        pf.FieldSystem((64, 1, 1), pf.UnitCell(1, "lamellar", 10.0))


def test_superseded_anderson_updater_fails_loudly():
    """The engine keeps one Anderson history per system: an AndersonUpdater whose system has
    since had another one set up raises instead of stepping with the other's history."""
    import types

    import polyfields as pf
    u1, u2 = pf.AndersonUpdater(nhist=5), pf.AndersonUpdater(nhist=5)
    sys_ = types.SimpleNamespace(_anderson=u2)
    u2._owns(sys_)
    with pytest.raises(RuntimeError, match="one Anderson history per system"):
        u1._owns(sys_)
    u1.system = sys_
    with pytest.raises(RuntimeError, match="one Anderson history per system"):
        u1.step()


def _declared_params():
    """{name: [parameter declarations]} of the header's entry points."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(pf_[a-z_0-9]+)\s*\(([^()]*)\)\s*;", text):
        params = params.strip()
        out[name] = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
    return out


def test_julia_shim_calls_match_the_header():
    """polyfields.jl_gb300/julia/PolyFieldsGPU.jl cannot run without Julia, so its ccalls are
    checked against the header statically: every symbol is declared, with as many arguments,
    pointers where the C side takes pointers and scalars where it takes scalars."""
    shim = open(os.path.join(ROOT, "polyfields.jl_gb300", "julia", "PolyFieldsGPU.jl")).read()
    calls = re.findall(r"ccall\(\(:(pf_[a-z_0-9]+),\s*lib\),\s*[\w{}]+,\s*\(([^()]*)\)", shim, flags=re.S)
    assert len(calls) >= 20
    decl = _declared_params()
    for name, types in calls:
        assert name in decl, name
        jt = [t.strip() for t in types.split(",") if t.strip()]
        assert len(jt) == len(decl[name]), (name, jt, decl[name])
        for j, c in zip(jt, decl[name]):
            j_ptr = j.startswith(("Ptr", "Ref", "Cstring"))
            assert j_ptr == ("*" in c), (name, j, c)


def test_julia_shim_structs_match_the_header():
    """The shim's PFOptions / PFResults mirror pf_scft_options / pf_scft_results field by field
    (same names, order and C types), so `Ref{PFOptions}` passes the layout the library reads."""
    shim = open(os.path.join(ROOT, "polyfields.jl_gb300", "julia", "PolyFieldsGPU.jl")).read()
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    ctype = {"Cint": "int", "Cdouble": "double"}
    for jname, cname in (("PFOptions", "pf_scft_options"), ("PFResults", "pf_scft_results")):
        body = re.search(r"struct " + jname + r"\b.*?\n(.*?)\nend", shim, flags=re.S).group(1)
        jf = re.findall(r"^\s*(\w+)::(\w+)", body, flags=re.M)
        cbody = re.search(r"typedef struct " + cname + r"\s*\{(.*?)\}", text, flags=re.S).group(1)
        cf = re.findall(r"^\s*(int|double)\s+(\w+)\s*;", cbody, flags=re.M)
        assert [(n, ctype[t]) for n, t in jf] == [(n, t) for t, n in cf], jname


def test_ctypes_signatures_match_the_header():
    """polyfields/_lib.py binds every entry point with the header's argument count, pointers
    where the C side takes pointers, and struct layouts equal to the C typedefs."""
    import ctypes

    from polyfields import _lib as L
    decl = _declared_params()
    assert sorted(L.SIGNATURES) == sorted(decl)
    for name, (_, args) in L.SIGNATURES.items():
        assert len(args) == len(decl[name]), (name, args, decl[name])
        for a, c in zip(args, decl[name]):
            is_ptr = a in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(a, "_type_") and a.__name__.startswith("LP_")
            assert is_ptr == ("*" in c), (name, a, c)
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    ctype = {ctypes.c_int: "int", ctypes.c_double: "double"}
    for cls, cname in ((L.ScftOptions, "pf_scft_options"), (L.ScftResults, "pf_scft_results")):
        cbody = re.search(r"typedef struct " + cname + r"\s*\{(.*?)\}", text, flags=re.S).group(1)
        cf = re.findall(r"^\s*(int|double)\s+(\w+)\s*;", cbody, flags=re.M)
        assert [(n, ctype[t]) for n, t in cls._fields_] == [(n, t) for t, n in cf], cname
