"""Parser of include/sbm_capi.h for the host-side binding tests: the
integer constants (#define and the field enum), the prototypes (base type,
pointer depth and name per parameter) and the members of the structs."""
import re

from conftest import ROOT

HDR = (ROOT / "include" / "sbm_capi.h").read_text()


def _split_top(s):
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


def c_text():
    return re.sub(r"/\*.*?\*/", "", HDR, flags=re.S)


def c_constants():
    text = c_text()
    vals = {m.group(1): int(m.group(2))
            for m in re.finditer(r"#define\s+(SBM_\w+)\s+(-?\d+)\b", text)}
    body = re.search(r"enum\s+sbm_field\s*\{(.*?)\}", text, re.S).group(1)
    n = 0
    for item in _split_top(body):
        m = re.match(r"(\w+)\s*(=\s*(-?\d+))?$", item.strip())
        if not m:
            continue
        if m.group(3) is not None:
            n = int(m.group(3))
        vals[m.group(1)] = n
        n += 1
    return vals


def c_param(p):
    p = re.sub(r"\bconst\b|\bstruct\b", " ", p)
    stars = p.count("*")
    toks = p.replace("*", " ").split()
    return toks[0], stars, toks[-1]


def c_functions():
    text = " ".join(re.sub(r"^\s*#.*$", "", c_text(), flags=re.M).split())
    funcs = {}
    for stmt in re.split(r"[;{}]", text):
        m = re.match(r"\s*[\w\s\*]*?\b(sbm_\w+)\s*\(([^()]*)\)\s*$", stmt)
        if not m:
            continue
        params = [] if m.group(2).strip() in ("", "void") else [
            c_param(p) for p in m.group(2).split(",")]
        funcs[m.group(1)] = params
    return funcs


def c_struct(name):
    text = c_text()
    body = re.search(r"typedef\s+struct\s+%s\s*\{(.*?)\}\s*%s\s*;" % (name, name), text,
                     re.S).group(1)
    fields = []
    for stmt in body.split(";"):
        stmt = stmt.strip()
        if not stmt:
            continue
        ctype, rest = stmt.split(None, 1)
        for item in rest.split(","):
            m = re.match(r"(\w+)\s*(\[(\w+)\])?$", item.strip())
            fields.append((m.group(1).lower(), ctype, m.group(3)))
    return fields


def c_prototypes():
    """{name: (return base type, return pointer depth, params)}."""
    text = " ".join(re.sub(r"^\s*#.*$", "", c_text(), flags=re.M).split())
    out = {}
    for stmt in re.split(r"[;{}]", text):
        m = re.match(r"\s*([\w\s\*]*?)\b(sbm_\w+)\s*\(([^()]*)\)\s*$", stmt)
        if not m or not m.group(1).strip():
            continue
        ret = re.sub(r"\bconst\b", " ", m.group(1))
        rstars = ret.count("*")
        rbase = ret.replace("*", " ").split()[-1]
        params = [] if m.group(3).strip() in ("", "void") else [
            c_param(p) for p in m.group(3).split(",")]
        out[m.group(2)] = (rbase, rstars, params)
    return out
