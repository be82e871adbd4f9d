"""CPU: the ISO_C_BINDING module fortran/dns3d_gpu.f90 (the reference-side
binding a Fortran driver adds) stays in sync with include/dns3d_capi.h.

No Fortran compiler exists on either machine, so the check is textual: every
bind(C) derived type has the C struct's fields in the same order with the
matching kinds (c_int = int, c_double = double, c_long_long = long long),
and every interface names a declared C function with the same number of
arguments, each passed the way the C prototype takes it (a scalar by value,
everything else through a pointer)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "fortran", "dns3d_gpu.f90")
HDR = os.path.join(ROOT, "include", "dns3d_capi.h")

KIND = {"c_int": "int", "c_double": "double", "c_long_long": "long long"}


def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _strip_f(text):
    return "\n".join(line.split("!", 1)[0] for line in text.splitlines())


def c_structs():
    t = _strip_c(open(HDR).read())
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\}\s*(\w+);", t, re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mm = re.match(r"(unsigned long long|long long|const char\*|double|int|\w+)\s+(.*)", decl)
            assert mm, decl
            for n in mm.group(2).split(","):
                fields.append((n.strip(), mm.group(1)))
        out[m.group(1)] = fields
    return out


def c_functions():
    t = _strip_c(open(HDR).read())
    out = {}
    for m in re.finditer(r"(?:int|const char\*)\s+(dns3d_\w+)\s*\(([^)]*)\)\s*;", t):
        params = [" ".join(p.split()) for p in m.group(2).split(",") if p.strip()]
        out[m.group(1)] = params
    return out


def f_types():
    t = _strip_f(open(F90).read())
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)end type", t, re.S):
        fields = []
        for line in m.group(2).splitlines():
            mm = re.match(r"\s*(integer|real)\((\w+)\)\s*::\s*(.*)", line)
            if mm:
                fields += [(n.strip(), KIND[mm.group(2)]) for n in mm.group(3).split(",")]
        out[m.group(1)] = fields
    return out


def f_functions():
    t = _strip_f(open(F90).read())
    out = {}
    for m in re.finditer(r"function (\w+)\(([^)]*)\) bind\(C\)\n(.*?)end function", t, re.S):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        decl = {}
        for line in m.group(3).splitlines():
            mm = re.match(r"\s*(type|integer|real|character)\(([^)]*)\)\s*(?:,\s*([\w(), ]*?))?\s*::\s*(.*)", line)
            if not mm:
                continue
            attrs = mm.group(3) or ""
            for n in mm.group(4).split(","):
                n = re.sub(r"\(.*\)", "", n).strip()
                decl[n] = (mm.group(1), mm.group(2), "value" in attrs)
        out[m.group(1)] = [(a, decl[a]) for a in args]
    return out


def test_derived_types_match_c_structs():
    cs, ft = c_structs(), f_types()
    assert set(ft) == {"dns3d_config", "dns3d_pi_state", "dns3d_diag"}
    for name, fields in ft.items():
        assert fields == cs[name], name


def test_interfaces_match_prototypes():
    cf, ff = c_functions(), f_functions()
    assert len(ff) >= 25
    for name, args in ff.items():
        assert name in cf, name
        params = cf[name]
        assert len(args) == len(params), (name, args, params)
        for (a, (ftype, fkind, by_value)), p in zip(args, params):
            c_ptr = "*" in p
            if by_value and ftype in ("integer", "real"):
                assert not c_ptr and p.split()[0] == KIND[fkind], (name, a, p)
            else:
                # c_ptr by value, or a variable passed by reference
                assert c_ptr, (name, a, p)


def test_five_step_subroutines_bound():
    ff = f_functions()
    for n in ("dns3d_compute_source_terms", "dns3d_viscous_step", "dns3d_solve_pressure",
              "dns3d_pressure_correction", "dns3d_apply_boundary_conditions"):
        assert n in ff
