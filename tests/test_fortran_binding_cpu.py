"""The Fortran module include/rflu_gpu.f90 against the C header
include/rflu_gpu.h, read as text (no Fortran compiler exists here or on the
GPU machine, so the binding is checked by rule): every BIND(C) derived type
repeats its C struct field for field (names and interoperable kinds, in
order); every function the header declares has an interface with the same
binding name, argument names in the same order, and for each argument the
kind and passing that the C declaration requires (VALUE for scalars and for
opaque handles, by reference for structs and output scalars, arrays or a
TYPE(C_PTR) VALUE for pointers to data); the integer constants agree."""
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
INC = os.path.join(HERE, "..", "include")

SCALAR_KIND = {"int": "INTEGER(C_INT)", "long long": "INTEGER(C_LONG_LONG)",
               "unsigned long long": "INTEGER(C_LONG_LONG)", "double": "REAL(C_DOUBLE)"}
HANDLES = ("rflu_gpu_ctx", "rflu_setup")


def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _c_decl(decl):
    """'const double *cv' -> ('double', 1, 'cv')"""
    decl = decl.replace("const ", " ").strip()
    m = re.match(r"^(.*?)([\s\*]+)(\w+)$", decl)
    base, stars, name = m.group(1).strip(), m.group(2), m.group(3)
    return " ".join(base.split()), stars.count("*"), name


def c_header():
    src = _strip_c(open(os.path.join(INC, "rflu_gpu.h")).read())
    structs = {}
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for stmt in body.split(";"):
            stmt = " ".join(stmt.split())
            if not stmt:
                continue
            m = re.match(r"^((?:const\s+)?(?:unsigned\s+)?(?:long\s+long|int|double|char|void|\w+))\s+(.*)$", stmt)
            base = m.group(1).replace("const ", "").strip()
            for d in m.group(2).split(","):
                d = d.strip()
                fields.append((d.lstrip("*"), base, d.count("*")))
        structs[name] = fields
    funcs = {}
    for stmt in src.split(";"):
        m = re.search(r"^[ \t]*([\w \t\*]+?)[ \t\*]*\b(rflu_\w+)\s*\(([^)]*)\)\s*$", stmt, flags=re.M)
        if not m:
            continue
        ret, name, args = m.group(1), m.group(2), m.group(3).strip()
        funcs[name] = (" ".join(ret.replace("const ", "").split()),
                       [] if args in ("", "void") else [_c_decl(a) for a in args.split(",")])
    consts = {k: int(v.strip("()")) for k, v in re.findall(r"#define\s+(RFLU_\w+)\s+(\(?-?\d+\)?)", src)}
    return structs, funcs, consts


def fortran_module():
    text = open(os.path.join(INC, "rflu_gpu.f90")).read()
    text = re.sub(r"!.*", "", text)
    text = re.sub(r"&\s*\n\s*", " ", text)  # continuation lines
    types = {}
    for name, body in re.findall(r"TYPE\s*,\s*BIND\(C\)\s*::\s*(\w+)(.*?)END\s+TYPE", text, flags=re.S | re.I):
        fields = []
        for line in body.strip().splitlines():
            kind, names = line.split("::")
            for n in names.split(","):
                fields.append((n.strip(), " ".join(kind.split()).upper()))
        types[name] = fields
    ifaces = {}
    for ret, name, args, bind, body in re.findall(
            r"(INTEGER\(C_INT\)|TYPE\(C_PTR\))\s+FUNCTION\s+(\w+)\s*\(([^)]*)\)\s*BIND\(C,\s*NAME='(\w+)'\)"
            r"(.*?)END\s+FUNCTION", text, flags=re.S | re.I):
        decl = {}
        for line in body.strip().splitlines():
            line = line.strip()
            if not line or line.upper().startswith("IMPORT"):
                continue
            attrs, names = line.split("::")
            attrs = [a.strip().upper() for a in re.split(r",(?![^(]*\))", attrs)]
            for n in re.split(r",(?![^(]*\))", names):
                n = n.strip()
                decl[n.split("(")[0].lower()] = {"kind": attrs[0], "value": "VALUE" in attrs, "array": "(" in n}
        arglist = [a.strip() for a in args.split(",") if a.strip()]
        ifaces[bind] = {"name": name, "ret": ret.upper(), "args": arglist, "decl": decl}
    consts = {k: int(v) for k, v in re.findall(r"(RFLU_\w+)\s*=\s*(-?\d+)", text)}
    return types, ifaces, consts


def test_derived_types_match_structs():
    structs, _, _ = c_header()
    types, _, _ = fortran_module()
    assert set(structs) == set(types), (set(structs) ^ set(types))
    for name, fields in structs.items():
        ff = types[name]
        assert [n.lower() for n, _, _ in fields] == [n.lower() for n, _ in ff], name
        for (n, base, stars), (_, kind) in zip(fields, ff):
            want = "TYPE(C_PTR)" if stars else SCALAR_KIND[base]
            assert kind == want, (name, n, kind, want)


def _expected(base, stars, structs):
    """Acceptable (kind, value) pairs of a C parameter in a BIND(C) interface."""
    if base in HANDLES:
        return {("TYPE(C_PTR)", stars == 1)}
    if base in structs:
        assert stars == 1
        return {("TYPE(%s)" % base.upper(), False)}
    if stars == 0:
        return {(SCALAR_KIND[base], True)}
    if base == "void":
        return {("TYPE(C_PTR)", True)}
    return {(SCALAR_KIND[base], False), ("TYPE(C_PTR)", True)}


def test_every_function_has_a_matching_interface():
    structs, funcs, _ = c_header()
    _, ifaces, _ = fortran_module()
    assert len(funcs) >= 30
    assert set(funcs) == set(ifaces), set(funcs) ^ set(ifaces)
    for name, (ret, args) in funcs.items():
        f = ifaces[name]
        assert f["name"].lower() == name
        assert f["ret"] == ("INTEGER(C_INT)" if ret == "int" else "TYPE(C_PTR)"), name
        assert [a.lower() for a in f["args"]] == [n.lower() for _, _, n in args], name
        for base, stars, n in args:
            d = f["decl"][n.lower()]
            got = (d["kind"], d["value"])
            assert got in _expected(base, stars, structs), (name, n, got)
            if d["array"]:
                assert stars == 1 and not d["value"], (name, n)


def test_constants_agree():
    _, _, cc = c_header()
    _, _, fc = fortran_module()
    assert fc, "no constants parsed"
    for k, v in fc.items():
        assert cc[k] == v, k
    for k in ("RFLU_OK", "RFLU_ERR_STATE", "RFLU_EVENT_NAN", "RFLU_PREC_MIXED", "RFLU_BC_SLIPWALL", "RFLU_OPT_UNTILED"):
        assert k in fc


@pytest.mark.parametrize("name", ["rflu_grid_desc", "rflu_num_desc"])
def test_python_binding_structs_match_header(name):
    """The ctypes structures of rocflu_gb300.gpu follow the same field order."""
    from rocflu_gb300 import gpu

    structs, _, _ = c_header()
    cls = {"rflu_grid_desc": gpu.GridDesc, "rflu_num_desc": gpu.NumDesc}[name]
    assert [f for f, _ in cls._fields_] == [n for n, _, _ in structs[name]]
