"""The Fortran ISO_C_BINDING module include/sbm_capi.f90 against the C header
include/sbm_capi.h, without a Fortran compiler (neither machine has one):
every named constant has the header's value, both BIND(C) derived types
have the C structs' members in the same order and kinds, and every
interface names a declared function with the same arity and a matching
passing convention per argument (VALUE scalars <-> C values, by-reference
arguments <-> C pointers, TYPE(C_PTR) VALUE <-> a C pointer)."""
import re

import pytest

from capi_header import c_constants as _c_constants
from capi_header import c_functions as _c_functions
from capi_header import c_struct as _c_struct
from conftest import ROOT

F90 = (ROOT / "include" / "sbm_capi.f90").read_text()

# Fortran kind -> C base type
KIND = {"INTEGER(C_INT)": "int", "REAL(C_DOUBLE)": "double", "REAL(C_FLOAT)": "float",
        "INTEGER(C_SIZE_T)": "size_t", "INTEGER(C_INT64_T)": "int64_t",
        "INTEGER(C_INT16_T)": "int16_t", "CHARACTER(KIND=C_CHAR)": "char",
        "TYPE(SBM_PARAMS)": "sbm_params", "TYPE(SBM_SCALARS)": "sbm_scalars"}


def _f90_lines():
    out, buf = [], ""
    for raw in F90.splitlines():
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if s.startswith("&"):
            s = s[1:].strip()
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        out.append(buf + s)
        buf = ""
    return out


def _split_top(s):
    """Splits on commas outside parentheses."""
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur.strip())
    return parts


def _decl(line):
    """'KIND, ATTR :: a, b(*)' -> (kind, attrs, [(name, dim)])."""
    left, right = line.split("::", 1)
    attrs = [a.strip().upper() for a in _split_top(left)]
    names = []
    for item in _split_top(right):
        m = re.match(r"(\w+)\s*(\((.*)\))?$", item.strip())
        names.append((m.group(1).lower(), m.group(3)))
    return attrs[0].replace(" ", ""), attrs[1:], names


def _f90_types():
    types, cur = {}, None
    for line in _f90_lines():
        u = line.upper()
        m = re.match(r"TYPE\s*,\s*BIND\(C\)\s*::\s*(\w+)", u)
        if m:
            cur = m.group(1).lower()
            types[cur] = []
            continue
        if u.startswith("END TYPE"):
            cur = None
            continue
        if cur is not None:
            kind, _, names = _decl(line)
            for nm, dim in names:
                types[cur].append((nm, KIND[kind], dim))
    return types


def _f90_interfaces():
    funcs, cur = {}, None
    for line in _f90_lines():
        m = re.match(r"INTEGER\(C_INT\)\s+FUNCTION\s+(\w+)\s*\(([^)]*)\)\s*BIND\(C,\s*NAME='(\w+)'\)",
                     line, re.I)
        if m:
            args = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
            cur = {"name": m.group(1), "cname": m.group(3), "args": args, "decl": {}}
            funcs[m.group(3)] = cur
            continue
        if re.match(r"END\s+FUNCTION", line, re.I):
            cur = None
            continue
        if cur is not None and "::" in line and not line.strip().upper().startswith("IMPORT"):
            kind, attrs, names = _decl(line)
            for nm, dim in names:
                cur["decl"][nm] = (kind, "VALUE" in attrs, dim)
    return funcs


def _f90_constants():
    vals = {}
    for line in _f90_lines():
        if "PARAMETER" not in line.upper() or "::" not in line:
            continue
        for item in _split_top(line.split("::", 1)[1]):
            name, val = (x.strip() for x in item.split("="))
            vals[name.upper()] = int(val)
    return vals


def test_constants_match_the_header():
    c = _c_constants()
    f = _f90_constants()
    assert len(f) >= 30
    for name, val in f.items():
        assert name in c, name
        assert c[name] == val, (name, val, c[name])
    # every field id of the header is available to a Fortran host
    fields = [k for k in c if k.startswith("SBM_F_") and k != "SBM_F_COUNT"]
    assert fields and all(k in f for k in fields)


@pytest.mark.parametrize("name", ["sbm_params", "sbm_scalars"])
def test_derived_types_match_the_structs(name):
    f = _f90_types()[name]
    c = _c_struct(name)
    assert [(n, t) for n, t, _ in f] == [(n, t) for n, t, _ in c]
    for (_, _, fd), (_, _, cd) in zip(f, c):
        assert (fd or None) == (cd or None)


def test_interfaces_match_the_prototypes():
    cfun = _c_functions()
    ffun = _f90_interfaces()
    assert len(ffun) >= 20
    for cname, fi in ffun.items():
        assert fi["name"].lower() == cname.lower()
        assert cname in cfun, cname
        params = cfun[cname]
        assert len(params) == len(fi["args"]), cname
        for arg, (cbase, stars, _) in zip(fi["args"], params):
            kind, value, _ = fi["decl"][arg]
            if kind == "TYPE(C_PTR)":
                assert stars == (1 if value else 2), (cname, arg)
            elif value:
                assert stars == 0 and cbase == KIND[kind], (cname, arg, cbase, stars)
            else:
                assert stars == 1 and cbase == KIND[kind], (cname, arg, cbase, stars)


def test_the_checks_catch_planted_mistakes(monkeypatch):
    import sys

    me = sys.modules[__name__]
    by_ref = F90.replace("INTEGER(C_INT), VALUE :: ny, nx, nz", "INTEGER(C_INT) :: ny, nx, nz", 1)
    assert by_ref != F90
    monkeypatch.setattr(me, "F90", by_ref)
    with pytest.raises(AssertionError):
        test_interfaces_match_the_prototypes()
    wrong = F90.replace("SBM_PC_LEARNED = 2", "SBM_PC_LEARNED = 3", 1)
    assert wrong != F90
    monkeypatch.setattr(me, "F90", wrong)
    with pytest.raises(AssertionError):
        test_constants_match_the_header()
