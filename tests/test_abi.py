"""The C-ABI library loads and exports exactly what include/hermes_gb300.h
declares; host-only entry points answer without a GPU."""
import ctypes as C
import os
import re

import pytest

from hermeshd_gb300 import _lib, config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "hermes_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(hermes_\w+)\s*\(", src, flags=re.M))


def test_header_and_binding_agree():
    assert header_functions() == set(_lib.EXPORTS)


def _header_struct_fields(name):
    src = open(os.path.join(ROOT, "include", "hermes_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if decl:
            typ, names = decl.split(None, 1)
            fields += [(n.strip(), typ) for n in names.split(",")]
    return fields


@pytest.mark.parametrize("cname,pycls", [("hermes_launch", "HermesLaunch"), ("hermes_output_units", "HermesOutputUnits")])
def test_small_structs_match_header(cname, pycls):
    """Field names and order of the ctypes mirrors of the header's small
    structs (their sizes are not reported by the library)."""
    fields = _header_struct_fields(cname)
    py = getattr(_lib, pycls)._fields_
    assert [f for f, _ in fields] == [f for f, _ in py]
    ctype = {"int32_t": C.c_int32, "double": C.c_double}
    assert [ctype[t] for _, t in fields] == [t for _, t in py]


def test_library_exports_every_symbol(hermes_lib):
    for name in _lib.EXPORTS:
        assert hasattr(hermes_lib, name), name


def test_abi_version_and_config_layout(hermes_lib):
    assert hermes_lib.hermes_abi_version() == _lib.ABI_VERSION == 8
    assert hermes_lib.hermes_config_size() == C.sizeof(_lib.HermesConfig)


@pytest.mark.parametrize("nb,nq", [(4, 2), (8, 2), (10, 3)])
def test_sizes(hermes_lib, nb, nq):
    cfg = config.Config(nx=7, ny=5, nz=3, nbasis=nb, iquad=nq, xlobc="wall", xhibc="wall")
    qe, sb = C.c_size_t(), C.c_size_t()
    assert hermes_lib.hermes_sizes(C.byref(_lib.to_c(cfg)), C.byref(qe), C.byref(sb)) == 0
    assert qe.value == 7 * 5 * 3 * 11 * nb
    nf = nq * nq
    faces = (8 * 5 * 3) + (7 * 5 * 3) + (7 * 5 * 3)      # x has nx+1 planes (walls); y, z periodic
    assert sb.value == faces * 11 * nf * 8


def test_bad_config_rejected_without_gpu(hermes_lib):
    cfg = _lib.to_c(config.Config(nbasis=27, iquad=3))
    ctx = C.c_void_p()
    assert hermes_lib.hermes_create(C.byref(cfg), None, C.byref(ctx)) == 1   # HERMES_ERR_CONFIG
    cfg = _lib.to_c(config.Config(nx=0))
    assert hermes_lib.hermes_create(C.byref(cfg), None, C.byref(ctx)) == 1
    assert not ctx.value


def test_empty_and_malformed_inputs_rejected_without_gpu(hermes_lib):
    """An ensemble of no boxes, a box with no cells, unknown boundary codes."""
    import numpy as np
    cfg = _lib.to_c(config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2))
    ctx = C.c_void_p()
    assert hermes_lib.hermes_ensemble_create(C.byref(cfg), 0, None, None, None, None, C.byref(ctx)) == 8
    dims = np.array([4, 0, 1], dtype=np.int32)
    assert hermes_lib.hermes_ensemble_create(C.byref(cfg), 1, dims.ctypes.data_as(C.POINTER(C.c_int32)), None, None,
                                             None, C.byref(ctx)) == 1
    bad = _lib.to_c(config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2))
    bad.bc[3] = 9
    assert hermes_lib.hermes_create(C.byref(bad), None, C.byref(ctx)) == 1
    bad.bc[3] = 4       # inflow is an x-low boundary only
    assert hermes_lib.hermes_create(C.byref(bad), None, C.byref(ctx)) == 1


def _header_prototypes():
    """name -> (return type text, [parameter type texts]) of every function
    the header declares."""
    src = open(os.path.join(ROOT, "include", "hermes_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*((?:const\s+)?[\w]+\s*\**)\s*(hermes_\w+)\s*\(([^)]*)\)\s*;", src, flags=re.M):
        params = [p.strip() for p in m.group(3).replace("\n", " ").split(",")]
        params = [] if params == ["void"] or params == [""] else params
        types = [re.sub(r"\b\w+\s*$", "", p).strip() if not p.endswith("*") else p for p in params]
        out[m.group(2)] = (m.group(1).strip(), types)
    return out


def _kind_c(t):
    if "*" in t:
        return "ptr"
    # size_t is uint64_t on the LP64 hosts this builds for (and ctypes.c_size_t is c_uint64 there)
    return {"int": "i32", "int32_t": "i32", "uint32_t": "u32", "uint64_t": "u64", "double": "f64",
            "size_t": "u64"}[t.replace("const", "").strip()]


def _kind_ctypes(t):
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    return {C.c_int32: "i32", C.c_uint32: "u32", C.c_uint64: "u64", C.c_double: "f64", C.c_size_t: "u64"}[t]


def test_ctypes_signatures_match_the_header(hermes_lib):
    """Every function the Python binding declares has the header's number of
    parameters and the same kind of each (pointer, 32/64-bit integer,
    double) and of its result: a mismatch would pass wrong values through
    ctypes without an error."""
    protos = _header_prototypes()
    L = _lib.lib()
    checked = 0
    for name, (ret, params) in protos.items():
        f = getattr(L, name)
        if f.argtypes is None:
            continue
        assert len(f.argtypes) == len(params), (name, params, f.argtypes)
        assert [_kind_ctypes(a) for a in f.argtypes] == [_kind_c(p) for p in params], name
        assert _kind_ctypes(f.restype) == _kind_c(ret), (name, ret, f.restype)
        checked += 1
    assert checked >= 30


def test_fortran_binding_matches_the_config_struct():
    """The ISO_C_BINDING mirror of hermes_config that INTEGRATION.md gives a
    Fortran driver has the header's fields in the header's order, each of the
    same width (uint64_t seed as c_int64_t: Fortran has no unsigned kinds)."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    body = re.search(r"type, bind\(C\) :: hermes_config\n(.*?)\n\s*end type", doc, flags=re.S).group(1)
    fort = []
    for line in body.splitlines():
        kind, names = line.split("::")
        kind = {"integer(c_int32_t)": "i32", "integer(c_int64_t)": "i64", "real(c_double)": "f64"}[kind.strip()]
        for n in names.split(","):
            n = n.strip()
            m = re.match(r"(\w+)\((\d+)\)", n)
            fort += [(m.group(1), kind)] * int(m.group(2)) if m else [(n, kind)]
    width = {"int32_t": "i32", "uint64_t": "i64", "double": "f64"}
    head = []
    for name, typ in _header_struct_fields("hermes_config"):
        m = re.match(r"(\w+)\[(\d+)\]", name)
        head += [(m.group(1), width[typ])] * int(m.group(2)) if m else [(name, width[typ])]
    assert fort == head


def test_fortran_interfaces_match_the_prototypes():
    """The Fortran interface blocks in INTEGRATION.md bind the header's
    functions with the header's number of arguments."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    protos = _header_prototypes()
    found = re.findall(r"function (hermes_\w+)\(([^)]*)\) bind\(C, name=\"(hermes_\w+)\"\)", doc)
    assert len(found) >= 3
    for fname, args, cname in found:
        assert fname == cname
        assert len([a for a in args.split(",") if a.strip()]) == len(protos[cname][1]), cname


def test_integration_python_stub_uses_the_binding():
    """The ctypes stub INTEGRATION.md shows a maintainer compiles and names
    only functions the binding exports."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    code = re.search(r"```python\n(.*?)```", doc, flags=re.S).group(1)
    compile(code, "INTEGRATION.md", "exec")
    used = set(re.findall(r"\b(hermes_\w+)\(", code))
    assert used and used <= set(_lib.EXPORTS)
    assert all(hasattr(_lib, n) for n in re.findall(r"_lib\.(\w+)\(", code))


def test_readme_examples_name_real_calls():
    """The README's Python examples compile, and the methods they call on the
    front end and the solver exist."""
    from hermeshd_gb300 import adjoint, hermeshd, solver
    doc = open(os.path.join(ROOT, "README.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", doc, flags=re.S)
    assert len(blocks) >= 3
    for b in blocks:
        compile(b, "README.md", "exec")
    text = "\n".join(blocks)
    for m in re.findall(r"\bhermeshd\.(\w+)\(", text):
        assert hasattr(hermeshd.Hermeshd, m), m
    for m in re.findall(r"\bs\.(\w+)\(", text):
        assert hasattr(solver.Solver, m), m
    for m in re.findall(r"\bfrom hermeshd_gb300\.adjoint import ([\w, ]+)", text):
        for n in m.split(","):
            assert hasattr(adjoint, n.strip()), n
