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


FORTRAN = os.path.join(ROOT, "mwf_gb300", "fortran")


def _fortran(name):
    """Source of a Fortran file of the drop-in, without comment lines and trailing comments."""
    lines = []
    for ln in open(os.path.join(FORTRAN, name)).read().splitlines():
        ln = ln.split("!")[0] if not ln.lstrip().startswith("#") else ""
        if ln.strip():
            lines.append(ln.rstrip())
    return "\n".join(lines)


def test_run_desc_layouts_agree():
    """The run descriptor of the C header, the ctypes mirror and the Fortran bind(c) type of
    mwf_gpu_c.f90 have the same members in the same order with the same C types, so a Fortran
    or Python caller passes exactly the struct the library reads."""
    from mwf_gb300 import _lib
    c = _c_struct_fields()
    assert len(c) == 21
    py = [(("double" if t is ctypes.c_double else "int"), n) for n, t in _lib.RunDescC._fields_]
    assert py == c
    src = _fortran("mwf_gpu_c.f90")
    ftype = re.search(r"type, bind\(c\) :: mwf_run_desc\n(.*?)\n\s*end type", src, flags=re.S).group(1)
    fort = []
    for kind, names in re.findall(r"(integer\(c_int\)|real\(c_double\))\s*::\s*([^\n]+)", ftype):
        for n in names.split(","):
            fort.append(("int" if kind.startswith("integer") else "double", n.split("=")[0].strip()))
    assert [t for t, _ in fort] == [t for t, _ in c]
    assert [n.lower() for _, n in fort] == [n.lower() for _, n in c]


C_SCALAR_KIND = {"double": "real(c_double)", "int": "integer(c_int)", "long long": "integer(c_long_long)",
                 "size_t": "integer(c_size_t)"}


def _c_prototypes():
    """name -> list of (is_pointer, scalar type) of the parameters declared in include/mwf_gpu.h."""
    src = open(os.path.join(ROOT, "include", "mwf_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(?:int|long long)\s+(mwf_\w+)\s*\(([^)]*)\)\s*;", src):
        ps = [p.strip() for p in params.split(",") if p.strip() and p.strip() != "void"]
        kinds = []
        for p in ps:
            base = ("double" if re.search(r"\bdouble\b", p) else "long long" if "long long" in p
                    else "size_t" if "size_t" in p else "int" if re.search(r"\bint\b|\bunsigned\b", p) else "other")
            kinds.append(("*" in p, base))
        out[name] = kinds
    return out


def _fortran_interfaces():
    """name -> (dummy names, {dummy: (Fortran type, by value)}) of mwf_gpu_c.f90's interface block."""
    src = _fortran("mwf_gpu_c.f90")
    block = re.search(r"\n\s*interface\n(.*?)\n\s*end interface", src, flags=re.S).group(1)
    funcs = re.findall(r"function (mwf_\w+)\(([^)]*)\)\s*&?\s*bind\(c, name='(mwf_\w+)'\)\n(.*?)end function",
                       re.sub(r"&\n\s*", " ", block), flags=re.S)
    out = {}
    for name, args, cname, decls in funcs:
        assert name == cname, name
        dummies = [a.strip() for a in args.split(",") if a.strip()]
        attrs = {}
        for decl in decls.split("\n"):
            m = re.match(r"\s*(type\(c_ptr\)|type\(\w+\)|integer\(c_\w+\)|real\(c_double\)|character\(kind=c_char\))"
                         r"([^:]*)::\s*(.+)", decl)
            if not m:
                continue
            for v in re.sub(r"\([^)]*\)", "", m.group(3)).split(","):   # drop array bounds
                attrs[re.match(r"\s*(\w+)", v).group(1)] = (m.group(1), "value" in m.group(2))
        out[cname] = (dummies, attrs)
    return out


def test_fortran_interfaces_match_header():
    """Every function of the Fortran interface module binds a header function with the same
    number of arguments; C pointers are passed by reference or as type(c_ptr), value; C scalars
    by value with the matching kind."""
    protos = _c_prototypes()
    funcs = _fortran_interfaces()
    assert len(funcs) >= 17
    for cname, (dummies, attrs) in funcs.items():
        assert cname in protos, cname
        c = protos[cname]
        assert len(dummies) == len(c), cname
        for d, (is_ptr, base) in zip(dummies, c):
            ftype, by_value = attrs[d]
            if is_ptr:
                assert (ftype == "type(c_ptr)" and by_value) or not by_value, (cname, d)
            else:
                assert by_value and ftype != "type(c_ptr)", (cname, d)
                assert ftype == C_SCALAR_KIND[base], (cname, d, ftype, base)


# The reference's public names that main.f90, io.f90, turb.f90 and the utilities use: the
# velocity module's variables and procedures (program/velocity.f90:15-17, 21-180) and the
# transform module's procedures (program/transform.fftw5.f90:33, 64, 122).
VELOCITY_VARIABLES = ["vel_p", "vel_c", "vel_c2", "vel_onl", "vel_nl", "lhs", "rhs", "nst"]
VELOCITY_PROCEDURES = ["vel_TS", "vel_precompute", "vel_clk_time", "vel_imposesym", "vel_addlam", "vel_mpt2phys",
                       "epos", "eposC", "vel_energy", "vel_history"]
TRANSFORM_PROCEDURES = ["tra_precompute", "tra_spec2phys", "tra_phys2spec"]


def _module_names(src, module):
    body = re.search(r"\bmodule %s\n(.*?)\nend module %s" % (module, module), src, flags=re.S | re.I).group(1)
    head, _, procs = body.partition("\ncontains")
    variables = set()
    for attrs, decl in re.findall(r"^[ \t]*((?:type[ \t]*\(\w+\)|logical|integer|double precision)[^:\n]*)::[ \t]*(.+)$",
                                  head, flags=re.M):
        if "private" in attrs:
            continue
        for v in re.sub(r"\([^)]*\)", "", decl).split(","):
            variables.add(v.split("=")[0].strip().lower())
    heads = re.findall(r"^[ \t]*(?:[\w()]+[ \t]+)*?(?:subroutine|function)[ \t]+(\w+)", procs, flags=re.M | re.I)
    return variables, {h.lower() for h in heads}


def test_velocity_module_keeps_the_reference_names():
    src = _fortran("velocity.gpu.f90")
    variables, procs = _module_names(src, "velocity")
    for v in VELOCITY_VARIABLES:
        assert v.lower() in variables, v
    for p in VELOCITY_PROCEDURES:
        assert p.lower() in procs, p
    private = re.findall(r"^\s*(?:type\(c_ptr\)|logical), private :: (\w+)", src, flags=re.M)
    assert set(private) == {"vel_h", "vel_host_newer"}


def test_transform_module_keeps_the_reference_names():
    _, procs = _module_names(_fortran("transform.cuda.f90"), "transform")
    for p in TRANSFORM_PROCEDURES:
        assert p.lower() in procs, p


def test_fortran_modules_call_only_bound_functions():
    """Every library function the two modules call is bound in mwf_gpu_c.f90 (and so declared in
    the header, by test_fortran_interfaces_match_header)."""
    bound = set(_fortran_interfaces())
    for f in ("velocity.gpu.f90", "transform.cuda.f90"):
        called = set(re.findall(r"\b(mwf_\w+)\s*\(", _fortran(f))) - {"mwf_check", "mwf_run_desc"}
        assert called and called <= bound, (f, called - bound)
