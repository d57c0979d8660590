"""The Fortran side of the boundary (ads_mpi_gb300/fortran/ads_gpu.F90) against
the C-ABI it binds (include/ads_gpu.h), checked as text on the CPU: no Fortran
compiler exists on either machine, so a wrong ISO_C_BINDING interface would
otherwise only show in a user's build.  For every bind(c) function: the C
prototype exists, has the same number of arguments, and each argument passes
the same way (by value or by reference) with the same type and constness; the
bind(c) derived types match the C structs field by field; the integer
parameters equal the C macros."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "ads_mpi_gb300", "fortran", "ads_gpu.F90")
HDR = os.path.join(ROOT, "include", "ads_gpu.h")


def _strip_c_comments(s):
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def c_prototypes():
    s = _strip_c_comments(open(HDR).read())
    s = re.sub(r"#[^\n]*", " ", s)
    protos = {}
    for m in re.finditer(r"\b(int|const char\s*\*|void\s*\*|long long)\s+(ads_\w+)\s*\(([^)]*)\)\s*;", s):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        args = [a.strip() for a in args.split(",")] if args.strip() not in ("", "void") else []
        protos[name] = (re.sub(r"\s+", " ", ret), args)
    return protos


def c_structs():
    s = _strip_c_comments(open(HDR).read())
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \w+;", s, flags=re.S):
        fields = []
        for line in m.group(2).split(";"):
            line = line.strip()
            if line:
                ty, name = line.rsplit(None, 1)
                fields.append((ty.strip(), name.strip()))
        out[m.group(1)] = fields
    return out


def c_macros():
    s = open(HDR).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (ADS_\w+) (-?\d+)\b", s)}


def _f90_lines():
    text = open(F90).read()
    text = re.sub(r"&\s*\n\s*", " ", text)  # join continuation lines
    return [re.sub(r"!.*", "", l).rstrip() for l in text.splitlines()]


def f90_interfaces():
    """name -> (result type, [arg names], {arg: declaration})"""
    lines = _f90_lines()
    out = {}
    i = 0
    while i < len(lines):
        m = re.match(r"\s*(integer\(c_int\)|type\(c_ptr\))\s+function\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name=\"(\w+)\"\)",
                     lines[i])
        if m:
            res, _, args, cname = m.groups()
            names = [a.strip() for a in args.split(",") if a.strip()]
            decls = {}
            i += 1
            while not re.match(r"\s*end function", lines[i]):
                d = re.match(r"\s*(.+?)\s*::\s*(.+)", lines[i])
                if d and not d.group(1).startswith("import"):
                    for v in re.split(r",(?![^(]*\))", d.group(2)):
                        v = v.strip()
                        base = re.match(r"(\w+)", v).group(1)
                        decls[base] = (d.group(1).replace(" ", ""), "(" in v)
                i += 1
            out[cname] = (res, names, decls)
        i += 1
    return out


def f90_types():
    lines = _f90_lines()
    out = {}
    for i, l in enumerate(lines):
        m = re.match(r"\s*type,\s*bind\(c\)\s*::\s*(\w+)", l)
        if m:
            fields = []
            j = i + 1
            while not re.match(r"\s*end type", lines[j]):
                d = re.match(r"\s*(.+?)\s*::\s*(\w+)", lines[j])
                if d:
                    fields.append((d.group(1).replace(" ", ""), d.group(2)))
                j += 1
            out[m.group(1)] = fields
    return out


def f90_parameters():
    out = {}
    for l in _f90_lines():
        m = re.match(r"\s*integer\(c_int\),\s*parameter\s*::\s*(.+)", l)
        if m:
            for item in m.group(1).split(","):
                k, v = item.split("=")
                out[k.strip()] = int(v)
    return out


def _c_kind(arg):
    """(passing, type, const) of a C parameter declaration."""
    a = arg.replace("const ", "const@").strip()
    const = "const@" in a
    a = a.replace("const@", "")
    array = re.search(r"\[\s*\d*\s*\]\s*$", a) is not None
    a = re.sub(r"\[\s*\d*\s*\]\s*$", "", a)
    stars = a.count("*")
    base = a.replace("*", " ").split()[0]
    if base in ("ads_handle", "void") or stars >= 2:
        return ("value", "ptr", False) if base in ("ads_handle", "void") and stars == 1 else ("ref", "ptr", const)
    if stars == 1 or array:
        return ("ref", base, const)
    return ("value", base, False)


_F2C = {"integer(c_int)": "int", "real(c_double)": "double", "character(kind=c_char)": "char",
        "type(ads_opts)": "ads_opts", "type(ads_stats)": "ads_stats"}


def _f_kind(decl):
    ty, _ = decl
    parts = ty.split(",")
    base = parts[0]
    attrs = parts[1:]
    if base == "type(c_ptr)":
        return ("value", "ptr", False) if "value" in attrs else ("ref", "ptr", False)
    kind = _F2C[base]
    if "value" in attrs:
        return ("value", kind, False)
    return ("ref", kind, "intent(in)" in attrs)


def test_every_fortran_binding_matches_its_c_prototype():
    protos = c_prototypes()
    ifaces = f90_interfaces()
    assert len(ifaces) >= 20
    for cname, (res, names, decls) in ifaces.items():
        assert cname in protos, cname
        cret, cargs = protos[cname]
        assert (res == "integer(c_int)") == (cret == "int"), cname
        assert len(names) == len(cargs), (cname, names, cargs)
        for fn, ca in zip(names, cargs):
            fk = _f_kind(decls[fn])
            ck = _c_kind(ca)
            if fk[1] == "ptr" and fk[0] == "value":
                # type(c_ptr), value: any C pointer (optional arrays, handles, buffers)
                assert ck[0] == "value" and ck[1] == "ptr" or ck[0] == "ref", (cname, fn, ca)
                continue
            assert fk[:2] == ck[:2], (cname, fn, ca, fk, ck)
            assert fk[2] == ck[2], ("constness", cname, fn, ca)


def test_fortran_binds_the_step_api():
    want = {"ads_default_opts", "ads_create", "ads_destroy", "ads_dims", "ads_qp_points", "ads_set_form",
            "ads_set_oil", "ads_get_drained", "ads_save_spline_plot", "ads_multistep", "ads_set_coeffs",
            "ads_get_coeffs", "ads_step", "ads_steps", "ads_get_stats", "ads_assemble", "ads_solve",
            "ads_apply_mass", "ads_heat_adjoint", "ads_heat_jvp", "ads_status_string"}
    assert want <= set(f90_interfaces())


def test_bind_c_types_match_the_c_structs():
    cs = c_structs()
    ft = f90_types()
    for name in ("ads_opts", "ads_stats"):
        assert name in ft and name in cs
        cf = [( _F2C_t(t), n) for t, n in cs[name]]
        ff = [(_F2C[t], n) for t, n in ft[name]]
        assert ff == cf, name


def _F2C_t(t):
    return {"int": "int", "double": "double"}[t]


def test_fortran_parameters_equal_the_c_macros():
    macros = c_macros()
    params = f90_parameters()
    assert params
    for k, v in params.items():
        assert k in macros and macros[k] == v, k
