"""The C-ABI library builds, loads and exports every symbol of include/mwf_gpu.h (CPU only)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "mwf_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mwf_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from mwf_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    from mwf_gb300 import _lib
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n


def test_host_only_entry_points(lib):
    import mwf_gb300 as mwf
    p = mwf.RunParams(K0=6, MM=512, NN=512)
    d = p.to_c()
    assert lib.mwf_run_dof(ctypes.byref(d)) == 11 * 1023 * 512
    assert mwf.footprint_bytes([p]) > 16 * 5 * 17 * 1536 * 512
    bad = mwf.RunParams(K0=4, MM=5, NN=8)   # 5 is not of the form 2^a 3^b
    assert mwf.footprint_bytes([bad]) == -1


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import mwf_gb300 as mwf
    with pytest.raises(mwf.MwfError) as e:
        mwf.Ensemble([mwf.RunParams()])
    assert e.value.code == -3


def _c_struct_fields():
    """(type, name) of mwf_run_desc's members in include/mwf_gpu.h, in order."""
    src = open(os.path.join(ROOT, "include", "mwf_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct mwf_run_desc \{(.*?)\} mwf_run_desc;", src, flags=re.S).group(1)
    return re.findall(r"\b(int|double)\s+(\w+)\s*;", body)


def test_run_desc_layouts_agree():
    """The run descriptor of the C header, the ctypes mirror and the Fortran bind(c) type shown
    in INTEGRATION.md have the same members in the same order with the same C types, so a
    Fortran or Python caller passes exactly the struct the library reads."""
    from mwf_gb300 import _lib
    c = _c_struct_fields()
    assert len(c) == 21
    py = [(("double" if t is ctypes.c_double else "int"), n) for n, t in _lib.RunDescC._fields_]
    assert py == c
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    ftype = re.search(r"type, bind\(c\) :: mwf_run_desc\n(.*?)\n\s*end type", doc, flags=re.S).group(1)
    fort = []
    for kind, names in re.findall(r"(integer\(c_int\)|real\(c_double\))\s*::\s*([^\n!]+)", ftype):
        for n in names.split(","):
            fort.append(("int" if kind.startswith("integer") else "double", n.split("=")[0].strip()))
    assert [t for t, _ in fort] == [t for t, _ in c]
    assert [n.lower() for _, n in fort] == [n.lower() for _, n in c]


def _c_prototypes():
    """name -> list of (is_pointer, base type) of the parameters declared in include/mwf_gpu.h."""
    src = open(os.path.join(ROOT, "include", "mwf_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, params in re.findall(r"\bint\s+(mwf_\w+)\s*\(([^)]*)\)\s*;", src):
        ps = [p.strip() for p in params.split(",") if p.strip() and p.strip() != "void"]
        out[name] = [("*" in p, "double" if re.search(r"\bdouble\b", p) else "int" if re.search(r"\bint\b", p)
                      else "other") for p in ps]
    return out


def test_fortran_interfaces_match_header():
    """Every function of the Fortran interface block in INTEGRATION.md binds a header function
    with the same number of arguments; C pointers are passed by reference or as type(c_ptr),
    value; C scalars by value with the matching kind."""
    protos = _c_prototypes()
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = re.search(r"\n  interface\n(.*?)\n  end interface", doc, flags=re.S).group(1)
    funcs = re.findall(r"function (mwf_\w+)\(([^)]*)\) bind\(c, name='(mwf_\w+)'\)\n(.*?)end function", block,
                       flags=re.S)
    assert len(funcs) >= 9
    for name, args, cname, decls in funcs:
        assert name == cname and cname in protos, name
        dummies = [a.strip() for a in args.split(",")]
        attrs = {}
        for decl in re.split(r"[;\n]", decls):
            m = re.match(r"\s*(type\(c_ptr\)|type\(\w+\)|integer\(c_int\)|real\(c_double\))([^:]*)::\s*(.+)", decl)
            if not m:
                continue
            for v in re.sub(r"\([^)]*\)", "", m.group(3)).split(","):   # drop array bounds
                var = re.match(r"\s*(\w+)", v).group(1)
                attrs[var] = (m.group(1), "value" in m.group(2))
        c = protos[cname]
        assert len(dummies) == len(c), name
        for d, (is_ptr, base) in zip(dummies, c):
            ftype, by_value = attrs[d]
            if is_ptr:
                assert (ftype == "type(c_ptr)" and by_value) or not by_value, (name, d)
            else:
                assert by_value and ftype != "type(c_ptr)", (name, d)
                assert ftype == ("real(c_double)" if base == "double" else "integer(c_int)"), (name, d)
