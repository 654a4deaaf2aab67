"""The Fortran host binding (bsam1.2_gb300/fortran/bsamgpu.f90) against the
C ABI (include/bsamg.h), checked without a Fortran compiler: every entry
point the header declares has exactly one BIND(C) interface of the same
name, with the same number of arguments, and each argument has the C kind
the header gives it (the Fortran type, and VALUE for a scalar passed by
value, by reference otherwise); the result kinds agree; every #define of the
header is a PARAMETER of the module with the same value.  The host module
(bsam_gpu_host.f90) calls only entry points the binding declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bsamg.h")
FDIR = os.path.join(ROOT, "bsam1.2_gb300", "fortran")


def c_prototypes():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"((?:const\s+)?\w+\s*\**)\s*\b(bsamg_\w+)\s*\(([^;]*?)\)\s*;", txt):
        params = [] if args.strip() in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (c_kind(ret.strip() + " x"), [c_kind(a) for a in params])
    return out


def c_kind(decl):
    d = " ".join(decl.replace("const", "").split())
    ref = "*" in d or "[" in d
    base = d.replace("*", " ").split("[")[0].split()[:-1]
    base = " ".join(base)
    if base in ("bsamg_ctx", "bsamg_hier", "void"):
        return ("ptr", "ref" if d.count("*") > 1 else "value")
    if base == "bsamg_qinit_fn":
        return ("funptr", "value")
    if base == "bsamg_regrid_params":
        return ("regrid", "ref")
    if base == "char":
        return ("ptr", "value") if decl.strip().endswith(" x") else ("char", "ref")
    kind = {"int": "int", "double": "double", "size_t": "size_t", "long long": "long long",
            "unsigned long long": "long long"}[base]
    return (kind, "ref" if ref else "value")


F_TYPES = {"INTEGER(C_INT)": "int", "REAL(C_DOUBLE)": "double", "INTEGER(C_SIZE_T)": "size_t",
           "INTEGER(C_LONG_LONG)": "long long", "TYPE(C_PTR)": "ptr", "TYPE(C_FUNPTR)": "funptr",
           "CHARACTER(KIND=C_CHAR)": "char", "TYPE(bsamg_regrid_params)": "regrid"}


def f_interfaces():
    txt = open(os.path.join(FDIR, "bsamgpu.f90")).read()
    txt = re.sub(r"!.*", "", txt)
    txt = re.sub(r"&\s*\n\s*", " ", txt)
    body = txt[txt.index("INTERFACE"):txt.index("END INTERFACE")]
    out = {}
    for m in re.finditer(r"FUNCTION\s+(\w+)\s*\(([^)]*)\)\s*BIND\(C,\s*NAME='(\w+)'\)\s*RESULT\((\w+)\)(.*?)END FUNCTION",
                         body, re.S):
        fname, args, cname, res, decls = m.groups()
        assert fname == cname, (fname, cname)
        names = [a.strip() for a in args.split(",") if a.strip()]
        kinds = {}
        for line in decls.splitlines():
            line = line.strip()
            if "::" not in line:
                continue
            spec, vars_ = line.split("::")
            attrs = [s.strip() for s in re.split(r",(?![^(]*\))", spec)]
            ftype = F_TYPES[attrs[0].replace(" ", "")]
            value = "VALUE" in attrs[1:]
            for v in re.split(r",(?![^(]*\))", vars_):
                v = v.strip()
                vname = v.split("(")[0].strip()
                kinds[vname] = (ftype, "value" if value else "ref")
        out[fname] = (kinds[res], [kinds[a] for a in names])
    return out


def equivalent(c, f):
    if c == f:
        return True
    # a C pointer the host passes as an opaque address (device arrays, user data)
    return c[1] == "ref" and c[0] in ("double", "int", "ptr") and f == ("ptr", "value")


def test_every_entry_point_has_a_matching_interface():
    cp, fi = c_prototypes(), f_interfaces()
    assert len(cp) > 40
    assert sorted(cp) == sorted(fi), (set(cp) ^ set(fi))
    for name, (cret, cargs) in cp.items():
        fret, fargs = fi[name]
        result = ("ptr", "value") if cret == ("char", "ref") else cret
        assert fret[0] == result[0], (name, cret, fret)
        assert len(cargs) == len(fargs), (name, len(cargs), len(fargs))
        for n, (ca, fa) in enumerate(zip(cargs, fargs)):
            assert equivalent(ca, fa), (name, n, ca, fa)


def test_every_constant_is_a_parameter():
    defines = dict(re.findall(r"#define (BSAMG_\w+) (-?\d+)", open(HEADER).read()))
    txt = re.sub(r"&\s*\n\s*", " ", re.sub(r"!.*", "", open(os.path.join(FDIR, "bsamgpu.f90")).read()))
    params = dict(re.findall(r"(BSAMG_\w+)\s*=\s*(-?\d+)", txt))
    assert defines and set(defines) <= set(params), set(defines) - set(params)
    for k, v in defines.items():
        assert params[k] == v, k


def test_regrid_params_type_matches_the_struct():
    txt = open(HEADER).read()
    cfields = re.search(r"typedef struct \{(.*?)\} bsamg_regrid_params;", txt, re.S).group(1)
    cf = [(t, n, int(k) if k else 1) for t, n, k in re.findall(r"(int|double)\s+(\w+)(?:\[(\d+)\])?;", cfields)]
    ftxt = open(os.path.join(FDIR, "bsamgpu.f90")).read()
    fbody = re.search(r"TYPE, BIND\(C\):: bsamg_regrid_params(.*?)END TYPE", ftxt, re.S).group(1)
    ff = []
    for spec, vars_ in re.findall(r"(INTEGER\(C_INT\)|REAL\(C_DOUBLE\)):: (.*)", fbody):
        for v in re.split(r",(?![^(]*\))", vars_):
            m = re.match(r"\s*(\w+)(?:\((\d+):(\d+)\))?", v)
            n = int(m.group(3)) - int(m.group(2)) + 1 if m.group(2) else 1
            ff.append(("int" if spec.startswith("INTEGER") else "double", m.group(1), n))
    assert cf == ff


def test_host_module_calls_declared_entry_points_only():
    txt = open(os.path.join(FDIR, "bsam_gpu_host.f90")).read()
    used = set(re.findall(r"\b(bsamg_\w+)\s*\(", re.sub(r"!.*", "", txt)))
    assert used and used <= set(f_interfaces()), used - set(f_interfaces())
    # the reference routines it replaces are cited
    for cite in ("afasroutines.f90:48-110", "bsamroutines.f90:682-702"):
        assert cite in txt, cite
