"""Interpreter for the Fortran 90 subset the reference's sources are written in.

TEST INFRASTRUCTURE ONLY.  The reference (Fortran 90 + MPI) cannot be compiled
here: there is no Fortran compiler on either machine.  This module executes
its source files statement by statement so that make_reference_golden.py can
record the reference's own results on small seeded inputs; the tests read
only those committed fixtures.  Nothing in the product imports it.

Semantics, those of a Fortran compiler that neither contracts nor reassociates
floating-point operations (no -ffast-math, no FMA contraction):

* kinds: INTEGER (Python int), REAL(KIND=4) (numpy.float32), REAL(KIND=8)
  (Python float / numpy.float64), LOGICAL, CHARACTER.  A real literal without
  a D exponent or a _8 kind is REAL(4), rounded once from its decimal text to
  binary32.  An operation on two kinds converts the lower one (INTEGER < REAL(4)
  < REAL(8)) first; INTEGER operations stay integer, `/` truncating toward
  zero.  Assignment converts to the variable's kind (rounding to nearest,
  truncation toward zero for INTEGER).
* every operation rounds once; x**n with an INTEGER exponent is evaluated by
  repeated squaring, the method of libgcc's __powidf2 that gfortran calls or
  inlines, so x**2 = x*x and x**3 = x*(x*x).
* array expressions are elementwise on numpy arrays (each element the scalar
  expression); the right-hand side is evaluated completely before it is
  stored; SUM accumulates sequentially in array-element (column-major)
  order; WHERE evaluates its mask once, before its assignments.
* EXP, LOG, TANH and real ** real come from the C library (Python's math
  module, i.e. the libm the compiled reference and the C oracle call), the
  REAL(4) versions (expf, ...) through ctypes; SQRT, ABS, MAX and MIN are
  exact operations.
* procedure arguments by reference: an array actual (whole, section or
  element) is copied in onto the dummy's explicit shape by sequence
  association (column-major) and copied back unless the dummy is
  INTENT(IN); a scalar variable actual is copied back likewise.
* subscripts are bounds-checked: an access outside a declared extent raises
  FortranError instead of aliasing other memory -- unless the Interp is made
  with bounds="linear", which addresses such an element of a rank-3 array by
  its column-major offset, as compiled code without bounds checks does.
* main-program arrays and ALLOCATE start as zeros (static storage and fresh
  pages); a procedure's automatic arrays and real scalars start as NaN, so
  that a value read before it is written shows in the results.
* MPI on one rank (MPI_ALLGATHER copies its send value into element 0 of the
  receive buffer); OPEN / READ / WRITE / PRINT go through hooks of the
  Interp object; INCLUDE 'mpif.h' defines the MPI constants used.

Statements covered: declarations (INTEGER, REAL, REAL(KIND=n), DOUBLE
PRECISION, LOGICAL, CHARACTER(LEN=n); DIMENSION, ALLOCATABLE, INTENT,
PARAMETER), DATA, ALLOCATE / DEALLOCATE, assignment, IF / ELSE IF / ELSE
(block and one-line), DO (counted and WHILE), EXIT, CYCLE, RETURN, WHERE /
ELSEWHERE (block and one-line), SELECT CASE, CALL, OPEN, CLOSE, READ, WRITE
(external and internal with (In) formats), PRINT.  Anything else raises
FortranError.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math
import re
from fractions import Fraction

import numpy as np

__all__ = ["FortranError", "Stop", "Interp", "FArr"]


class FortranError(RuntimeError):
    pass


class Stop(Exception):
    """Raised by a hook to end the program being run."""


I, R4, R8, L, CH = "I", "R4", "R8", "L", "CH"
_RANK = {I: 0, R4: 1, R8: 2}
_NP = {R4: np.float32, R8: np.float64, I: np.int64, L: np.bool_}

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _n, _na in (("expf", 1), ("logf", 1), ("tanhf", 1), ("powf", 2)):
    _f = getattr(_libm, _n)
    _f.restype = ctypes.c_float
    _f.argtypes = [ctypes.c_float] * _na


# ----------------------------------------------------------------- values
def kind_of(v):
    if isinstance(v, np.ndarray):
        c = v.dtype.kind
        if c == "f":
            return R8 if v.dtype.itemsize == 8 else R4
        if c == "b":
            return L
        if c in "iu":
            return I
        raise FortranError(f"array of dtype {v.dtype}")
    if isinstance(v, (bool, np.bool_)):
        return L
    if isinstance(v, np.float32):
        return R4
    if isinstance(v, float):
        return R8
    if isinstance(v, (int, np.integer)):
        return I
    if isinstance(v, str):
        return CH
    raise FortranError(f"value of type {type(v).__name__}")


def convert(v, k):
    if isinstance(v, np.ndarray):
        if k == R8:
            return v.astype(np.float64, copy=False)
        if k == R4:
            return v.astype(np.float32, copy=False)
        if k == I:
            return (np.trunc(v) if v.dtype.kind == "f" else v).astype(np.int64)
        if k == L:
            return v.astype(bool, copy=False)
        raise FortranError(f"array to kind {k}")
    if k == R8:
        return float(v)
    if k == R4:
        return np.float32(v)
    if k == I:
        return int(v)
    if k == L:
        return bool(v)
    if k == CH:
        return str(v)
    raise FortranError(f"conversion to kind {k}")


def f32_from_text(s: str) -> np.float32:
    """The binary32 value nearest the decimal literal s (ties to even)."""
    fr = Fraction(s)
    c = np.float32(float(fr))
    best, berr = c, abs(Fraction(float(c)) - fr)
    for cand in (np.nextafter(c, np.float32(-np.inf)), np.nextafter(c, np.float32(np.inf))):
        err = abs(Fraction(float(cand)) - fr)
        if err < berr or (err == berr and (int(cand.view(np.uint32)) & 1) == 0):
            best, berr = cand, err
    return np.float32(best)


def literal_value(text: str):
    t = text.upper()
    kind = None
    if "_" in t:
        t, ks = t.split("_", 1)
        kind = int(ks)
    if "D" in t:
        return float(t.replace("D", "E"))
    if "." in t or "E" in t:
        return float(t) if kind == 8 else f32_from_text(t)
    return int(t)


def _int_div(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        a, b = np.asarray(a, dtype=np.int64), np.asarray(b, dtype=np.int64)
        q = np.abs(a) // np.abs(b)
        return np.where((a >= 0) == (b >= 0), q, -q)
    if b == 0:
        raise FortranError("integer division by zero")
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def powi(x, n: int):
    """x**n for an INTEGER n by repeated squaring (libgcc __powidf2)."""
    m = -n if n < 0 else n
    y = x if m & 1 else None
    with np.errstate(all="ignore"):
        while True:
            m >>= 1
            if not m:
                break
            x = x * x
            if m & 1:
                y = x if y is None else y * x
        if y is None:
            y = np.ones_like(x) if isinstance(x, np.ndarray) else convert(1, kind_of(x))
        if n < 0:
            y = convert(1, kind_of(y)) / y
    return y


def _map(fn, x, dtype):
    return np.fromiter((fn(v) for v in x.flat), dtype=dtype, count=x.size).reshape(x.shape)


def _math1(name):
    f8 = getattr(math, name)
    f4 = getattr(_libm, name + "f")

    def g8(v):
        try:
            return f8(v)
        except (ValueError, OverflowError):  # libm's IEEE results where Python raises
            if name == "exp":
                return math.inf
            if name == "log" and v == 0.0:
                return -math.inf
            return float("nan")

    def f(x):
        k = kind_of(x)
        if k == I:
            raise FortranError(f"{name.upper()} of an INTEGER")
        if isinstance(x, np.ndarray):
            return _map(g8, x, np.float64) if k == R8 else _map(lambda v: f4(float(v)), x, np.float32)
        return g8(float(x)) if k == R8 else np.float32(f4(float(x)))

    return f


def _rpow(a, b, k):
    def p8(x, y):
        try:
            return math.pow(x, y)
        except (ValueError, OverflowError):
            return float("nan")

    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        a_, b_ = np.broadcast_arrays(np.asarray(a), np.asarray(b))
        out = np.empty(a_.shape, dtype=_NP[k])
        for idx in np.ndindex(a_.shape):
            out[idx] = p8(float(a_[idx]), float(b_[idx])) if k == R8 else _libm.powf(float(a_[idx]), float(b_[idx]))
        return out
    return p8(float(a), float(b)) if k == R8 else np.float32(_libm.powf(float(a), float(b)))


def arith(op, a, b):
    ka, kb = kind_of(a), kind_of(b)
    if op == "//":
        return str(a) + str(b)
    if ka == I and kb == I:
        if op == "+":
            return a + b
        if op == "-":
            return a - b
        if op == "*":
            return a * b
        if op == "/":
            return _int_div(a, b)
        return a ** b
    if ka not in _RANK or kb not in _RANK:
        raise FortranError(f"arithmetic on kinds {ka}, {kb}")
    if op == "**" and kb == I and not isinstance(b, np.ndarray):
        return powi(a, int(b))
    k = ka if _RANK[ka] >= _RANK[kb] else kb
    a, b = convert(a, k), convert(b, k)
    with np.errstate(all="ignore"):
        if op == "+":
            return a + b
        if op == "-":
            return a - b
        if op == "*":
            return a * b
        if op == "/":
            if not isinstance(a, np.ndarray) and not isinstance(b, np.ndarray) and b == 0:
                return _NP[k](a) / _NP[k](b)  # IEEE result, as compiled code gives
            return a / b
        return _rpow(a, b, k)


def relation(op, a, b):
    ka, kb = kind_of(a), kind_of(b)
    if ka == CH or kb == CH:
        n = max(len(a), len(b))
        a, b = a.ljust(n), b.ljust(n)
    else:
        k = ka if _RANK[ka] >= _RANK[kb] else kb
        a, b = convert(a, k), convert(b, k)
    with np.errstate(all="ignore"):
        r = {"==": lambda: a == b, "/=": lambda: a != b, "<": lambda: a < b,
             "<=": lambda: a <= b, ">": lambda: a > b, ">=": lambda: a >= b}[op]()
    return r if isinstance(r, np.ndarray) else bool(r)


def _logical(op, a, b=None):
    arr = isinstance(a, np.ndarray) or isinstance(b, np.ndarray)
    if op == "NOT":
        return np.logical_not(a) if arr else not a
    if op == "AND":
        return np.logical_and(a, b) if arr else (bool(a) and bool(b))
    if op == "OR":
        return np.logical_or(a, b) if arr else (bool(a) or bool(b))
    if op == "EQV":
        return np.equal(a, b) if arr else bool(a) == bool(b)
    return np.not_equal(a, b) if arr else bool(a) != bool(b)


def _sum(x):
    if not isinstance(x, np.ndarray):
        return x
    k = kind_of(x)
    if x.size == 0:
        return convert(0, k)
    if k in (R4, R8):
        return x.dtype.type(np.add.accumulate(x.ravel(order="F"), dtype=x.dtype)[-1])
    return int(x.sum())


def _sum_planes(x):
    """SUM of a rank-3 real array in the order of the C oracle's reductions:
    a sequential partial per plane of the last dimension (column-major
    within it), then the partials in sequence.  Only for showing that the
    order of the reductions is the one difference between two codes."""
    if not isinstance(x, np.ndarray) or x.ndim != 3 or kind_of(x) not in (R4, R8):
        return _sum(x)
    t = x.dtype.type(0)
    for k in range(x.shape[2]):
        plane = x[:, :, k].ravel(order="F")
        if plane.size:
            t = t + np.add.accumulate(plane, dtype=x.dtype)[-1]
    return x.dtype.type(t)


def _minmax(is_max):
    def f(*args):
        m = args[0]
        for b in args[1:]:
            km, kb = kind_of(m), kind_of(b)
            k = km if _RANK[km] >= _RANK[kb] else kb
            m, b = convert(m, k), convert(b, k)
            if isinstance(m, np.ndarray) or isinstance(b, np.ndarray):
                m = np.maximum(m, b) if is_max else np.minimum(m, b)
            else:
                m = (m if m >= b else b) if is_max else (m if m <= b else b)
        return m

    return f


def _sign(a, b):
    ka, kb = kind_of(a), kind_of(b)
    if ka == I and kb == I:
        if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
            return np.where(np.asarray(b) >= 0, np.abs(a), -np.abs(a))
        return abs(a) if b >= 0 else -abs(a)
    k = ka if _RANK[ka] >= _RANK[kb] else kb
    a, b = convert(a, k), convert(b, k)
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return np.copysign(np.abs(a), b).astype(_NP[k])
    r = math.copysign(abs(float(a)), float(b))
    return r if k == R8 else np.float32(r)


def _mod(a, b):
    if kind_of(a) == I and kind_of(b) == I:
        return arith("-", a, arith("*", _int_div(a, b), b))
    k = kind_of(a) if _RANK[kind_of(a)] >= _RANK[kind_of(b)] else kind_of(b)
    a, b = convert(a, k), convert(b, k)
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return np.fmod(a, b)
    r = math.fmod(float(a), float(b))
    return r if k == R8 else np.float32(r)


def _floor(x):
    if isinstance(x, np.ndarray):
        return np.floor(x).astype(np.int64)
    return math.floor(x)


def _nint(x):
    if isinstance(x, np.ndarray):
        return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)
    return int(math.copysign(math.floor(abs(float(x)) + 0.5), float(x)))


def _abs(x):
    return np.abs(x) if isinstance(x, np.ndarray) else abs(x)


def _sqrt(x):
    k = kind_of(x)
    if k == I:
        raise FortranError("SQRT of an INTEGER")
    with np.errstate(all="ignore"):
        if isinstance(x, np.ndarray):
            return np.sqrt(x)
        if k == R4:
            return np.float32(np.sqrt(x))
        return math.sqrt(x) if x >= 0 else float("nan")


INTRINSICS = {
    "SQRT": _sqrt, "DSQRT": _sqrt,
    "EXP": _math1("exp"), "DEXP": _math1("exp"),
    "LOG": _math1("log"), "DLOG": _math1("log"),
    "TANH": _math1("tanh"), "DTANH": _math1("tanh"),
    "ABS": _abs, "DABS": _abs, "IABS": _abs,
    "MAX": _minmax(True), "MIN": _minmax(False), "DMAX1": _minmax(True), "DMIN1": _minmax(False),
    "MOD": _mod, "INT": lambda x: convert(x, I), "NINT": _nint, "FLOOR": _floor,
    "DBLE": lambda x: convert(x, R8), "SNGL": lambda x: convert(x, R4),
    "REAL": lambda x, k=4: convert(x, R8 if k == 8 else R4), "FLOAT": lambda x: convert(x, R4),
    "SUM": _sum,
    "MAXVAL": lambda x: x.dtype.type(x.max()), "MINVAL": lambda x: x.dtype.type(x.min()),
    "SIGN": _sign, "DSIGN": _sign, "SIZE": lambda x: int(np.asarray(x).size),
    "TRIM": lambda s: s.rstrip(), "LEN": lambda s: len(s),
}


# ------------------------------------------------------------------ lexer
_DOTWORDS = "AND|OR|NOT|EQ|NE|LT|LE|GT|GE|EQV|NEQV|TRUE|FALSE"
_TOK = re.compile(
    r"(?P<ws>[ \t]+)"
    r"|(?P<num>(?:\d+\.(?!(?:" + _DOTWORDS + r")\.)\d*|\.\d+|\d+)(?:[ED][+-]?\d+)?(?:_\d+)?)"
    r"|(?P<dot>\.(?:" + _DOTWORDS + r")\.)"
    r"|(?P<name>[A-Z_][A-Z0-9_]*)"
    r"|(?P<str>'(?:[^']|'')*'|\"(?:[^\"]|\"\")*\")"
    r"|(?P<op>\*\*|//|==|/=|<=|>=|::|[-+*/<>(),:=%])",
    re.I,
)
_DOTMAP = {".EQ.": "==", ".NE.": "/=", ".LT.": "<", ".LE.": "<=", ".GT.": ">", ".GE.": ">="}


def tokenize(s: str):
    out, pos = [], 0
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise FortranError(f"cannot tokenize {s[pos:pos + 20]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        t = m.group()
        if kind == "ws":
            continue
        if kind == "str":
            q = t[0]
            out.append(("str", t[1:-1].replace(q + q, q)))
        elif kind == "dot":
            u = t.upper()
            if u in _DOTMAP:
                out.append(("op", _DOTMAP[u]))
            elif u in (".TRUE.", ".FALSE."):
                out.append(("bool", u == ".TRUE."))
            else:
                out.append(("op", u.strip(".")))
        elif kind == "name":
            out.append(("name", t.upper()))
        elif kind == "num":
            out.append(("num", t))
        else:
            out.append(("op", t))
    return out


def _strip_comment(line: str) -> str:
    q = None
    for i, c in enumerate(line):
        if q:
            if c == q:
                q = None
        elif c in "'\"":
            q = c
        elif c == "!":
            return line[:i]
    return line


def logical_lines(text: str):
    """(first physical line number, statement text) of each statement."""
    out, buf, start = [], "", None
    for no, raw in enumerate(text.splitlines(), 1):
        s = _strip_comment(raw.replace("\t", " ")).strip()
        if not s:
            continue
        if buf and s.startswith("&"):
            s = s[1:]
        cont = s.endswith("&")
        if cont:
            s = s[:-1]
        if not buf:
            start = no
        buf += " " + s
        if not cont:
            for part in _split_semicolons(buf):
                if part.strip():
                    out.append((start, part.strip()))
            buf = ""
    return out


def _split_semicolons(s):
    parts, q, cur = [], None, ""
    for c in s:
        if q:
            if c == q:
                q = None
        elif c in "'\"":
            q = c
        elif c == ";":
            parts.append(cur)
            cur = ""
            continue
        cur += c
    parts.append(cur)
    return parts


def _split_top(toks, sep=","):
    """Split a token list at depth-0 separators."""
    parts, cur, depth = [], [], 0
    for t in toks:
        if t == ("op", "("):
            depth += 1
        elif t == ("op", ")"):
            depth -= 1
        if depth == 0 and t == ("op", sep):
            parts.append(cur)
            cur = []
        else:
            cur.append(t)
    parts.append(cur)
    return parts


def _match_paren(toks, i):
    """Index of the ')' closing the '(' at toks[i]."""
    depth = 0
    for j in range(i, len(toks)):
        if toks[j] == ("op", "("):
            depth += 1
        elif toks[j] == ("op", ")"):
            depth -= 1
            if depth == 0:
                return j
    raise FortranError("unbalanced parentheses")


# ----------------------------------------------------------------- arrays
class FArr:
    """A Fortran array: numpy data in column-major order and lower bounds."""

    __slots__ = ("a", "lb", "kind")

    def __init__(self, a, lb, kind):
        self.a, self.lb, self.kind = a, tuple(lb), kind


def _idx(A, subs, name):
    idx = []
    for d, s in enumerate(subs):
        i = s - A.lb[d]
        if i < 0 or i >= A.a.shape[d]:
            raise FortranError(f"{name}: subscript {d + 1} = {s} outside {A.lb[d]}:{A.lb[d] + A.a.shape[d] - 1}")
        idx.append(i)
    return tuple(idx)


def _slices(A, subs, name):
    """subs: per dimension an int or (lo, hi, step) with None for defaults."""
    out = []
    for d, s in enumerate(subs):
        lb, n = A.lb[d], A.a.shape[d]
        if isinstance(s, tuple):
            lo, hi, st = s
            lo = lb if lo is None else lo
            hi = lb + n - 1 if hi is None else hi
            st = 1 if st is None else st
            if st <= 0:
                raise FortranError(f"{name}: non-positive section stride")
            if hi >= lo and (lo < lb or hi > lb + n - 1):
                raise FortranError(f"{name}: section {lo}:{hi} of dimension {d + 1} outside {lb}:{lb + n - 1}")
            out.append(slice(lo - lb, max(hi - lb + 1, lo - lb), st))
        else:
            i = s - lb
            if i < 0 or i >= n:
                raise FortranError(f"{name}: subscript {d + 1} = {s} outside {lb}:{lb + n - 1}")
            out.append(i)
    return tuple(out)


# ------------------------------------------------------------- expressions
class _Parser:
    """Recursive-descent parser from tokens to evaluator closures f(frame)."""

    def __init__(self, toks, unit):
        self.t, self.i, self.unit = toks, 0, unit

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def next(self):
        t = self.peek()
        self.i += 1
        return t

    def accept(self, *ops):
        t = self.peek()
        if t[0] == "op" and t[1] in ops:
            self.i += 1
            return t[1]
        return None

    def expect(self, op):
        if not self.accept(op):
            raise FortranError(f"expected {op!r} at {self.peek()} in {self.t}")

    def done(self):
        return self.i >= len(self.t)

    # precedence climbing, lowest first
    def expr(self):
        return self.eqv()

    def eqv(self):
        a = self.orx()
        while True:
            op = self.accept("EQV", "NEQV")
            if not op:
                return a
            b = self.orx()
            a = (lambda a, b, op: lambda fr: _logical(op, a(fr), b(fr)))(a, b, op)

    def orx(self):
        a = self.andx()
        while self.accept("OR"):
            b = self.andx()
            a = (lambda a, b: lambda fr: _logical("OR", a(fr), b(fr)))(a, b)
        return a

    def andx(self):
        a = self.notx()
        while self.accept("AND"):
            b = self.notx()
            a = (lambda a, b: lambda fr: _logical("AND", a(fr), b(fr)))(a, b)
        return a

    def notx(self):
        if self.accept("NOT"):
            a = self.notx()
            return lambda fr: _logical("NOT", a(fr))
        return self.rel()

    def rel(self):
        a = self.concat()
        op = self.accept("==", "/=", "<", "<=", ">", ">=")
        if op:
            b = self.concat()
            return lambda fr: relation(op, a(fr), b(fr))
        return a

    def concat(self):
        a = self.add()
        while self.accept("//"):
            b = self.add()
            a = (lambda a, b: lambda fr: arith("//", a(fr), b(fr)))(a, b)
        return a

    def add(self):
        sign = self.accept("+", "-")
        a = self.mult()
        if sign == "-":
            a = (lambda a: lambda fr: -a(fr))(a)
        while True:
            op = self.accept("+", "-")
            if not op:
                return a
            b = self.mult()
            a = (lambda a, b, op: lambda fr: arith(op, a(fr), b(fr)))(a, b, op)

    def mult(self):
        a = self.power()
        while True:
            op = self.peek()
            if op[0] == "op" and op[1] in ("*", "/"):
                self.i += 1
                b = self.power()
                a = (lambda a, b, op: lambda fr: arith(op, a(fr), b(fr)))(a, b, op[1])
            else:
                return a

    def power(self):
        a = self.primary()
        if self.accept("**"):
            b = self.power_operand()
            return lambda fr: arith("**", a(fr), b(fr))
        return a

    def power_operand(self):
        sign = self.accept("+", "-")
        b = self.power()
        if sign == "-":
            return lambda fr: -b(fr)
        return b

    def primary(self):
        kind, v = self.next()
        if kind == "num":
            c = literal_value(v)
            return lambda fr: c
        if kind == "str":
            return lambda fr: v
        if kind == "bool":
            return lambda fr: v
        if kind == "op" and v == "(":
            e = self.expr()
            self.expect(")")
            return e
        if kind == "op" and v in ("-", "+"):  # a sign after an operator (extension)
            a = self.power()
            return (lambda fr: -a(fr)) if v == "-" else a
        if kind == "name":
            if self.peek() == ("op", "("):
                self.i += 1
                args = self.arglist()
                return self.unit.designator_or_call(v, args)
            return self.unit.variable(v)
        raise FortranError(f"unexpected token {v!r} in {self.t}")

    def arglist(self):
        """Arguments up to the closing ')': each an expression, a section
        (lo, hi, step) of closures or None, or a keyword (name, expr)."""
        args = []
        if self.accept(")"):
            return args
        while True:
            if self.peek()[0] == "name" and self.peek(1) == ("op", "="):
                key = self.next()[1]
                self.next()
                args.append(("kw", key, self.expr()))
            else:
                args.append(self.subscript())
            if self.accept(")"):
                return args
            self.expect(",")

    def subscript(self):
        lo = hi = st = None
        if self.peek() != ("op", ":"):
            lo = self.expr()
            if self.peek() != ("op", ":"):
                return ("e", lo)
        self.expect(":")
        if self.peek() not in (("op", ","), ("op", ")"), ("op", ":")):
            hi = self.expr()
        if self.accept(":"):
            st = self.expr()
        return ("s", lo, hi, st)


def parse_expr(toks, unit):
    p = _Parser(toks, unit)
    e = p.expr()
    if not p.done():
        raise FortranError(f"trailing tokens {p.t[p.i:]}")
    return e


# ------------------------------------------------------------ declarations
class Decl:
    __slots__ = ("name", "kind", "clen", "dims", "alloc", "intent", "param", "init", "line")

    def __init__(self, name, kind, clen, dims, alloc, intent, param, init, line):
        self.name, self.kind, self.clen, self.dims = name, kind, clen, dims
        self.alloc, self.intent, self.param, self.init, self.line = alloc, intent, param, init, line


_TYPE_WORDS = ("INTEGER", "REAL", "DOUBLE", "LOGICAL", "CHARACTER")


def _type_spec(toks):
    """(kind, character length, index after the type spec)."""
    w = toks[0][1]
    i = 1
    clen = None
    if w == "DOUBLE":
        if toks[1] != ("name", "PRECISION"):
            raise FortranError("DOUBLE without PRECISION")
        return R8, None, 2
    kind = {"INTEGER": I, "REAL": R4, "LOGICAL": L, "CHARACTER": CH}[w]
    if i < len(toks) and toks[i] == ("op", "("):
        j = _match_paren(toks, i)
        inner = toks[i + 1:j]
        if inner and inner[0][0] == "name" and len(inner) > 1 and inner[1] == ("op", "="):
            inner = inner[2:]
        val = int(inner[0][1]) if len(inner) == 1 and inner[0][0] == "num" else None
        if kind == CH:
            clen = val
        elif kind == R4 and val == 8:
            kind = R8
        elif kind == R4 and val not in (4, None):
            raise FortranError(f"REAL kind {val}")
        i = j + 1
    elif i < len(toks) and toks[i] == ("op", "*"):
        val = int(toks[i + 1][1])
        if kind == R4 and val == 8:
            kind = R8
        if kind == CH:
            clen = val
        i += 2
    return kind, clen, i


def _dim_spec(toks, unit):
    """[(lo closure, hi closure)] or [None] per deferred dimension."""
    dims = []
    for part in _split_top(toks):
        if part == [("op", ":")]:
            dims.append(None)
            continue
        bits = _split_top(part, ":")
        if len(bits) == 1:
            dims.append((lambda fr: 1, parse_expr(bits[0], unit)))
        else:
            dims.append((parse_expr(bits[0], unit), parse_expr(bits[1], unit)))
    return dims


# -------------------------------------------------------------- program units
class Frame:
    __slots__ = ("v", "unit", "interp", "ovr")

    def __init__(self, unit, interp):
        self.v, self.unit, self.interp = {}, unit, interp
        self.ovr = interp.overrides.get(unit.name, {})


class _Ref:
    """An actual argument: get() its value, view() an array view, set(v)."""

    def __init__(self, get, view=None, set_=None):
        self.get, self.view, self.set = get, view, set_


MPI_CONSTS = {"MPI_COMM_WORLD": 0, "MPI_DOUBLE_PRECISION": 1, "MPI_STATUS_SIZE": 6}


class Unit:
    def __init__(self, name, kind, args, stmts, interp, path):
        self.name, self.kind, self.args, self.interp, self.path = name, kind, args, interp, path
        self.decls: dict[str, Decl] = {}
        self.data = []
        self.includes_mpi = False
        self.stmts = []  # (line, tokens) of the executable part
        for line, toks in stmts:
            if self._declaration(line, toks):
                continue
            self.stmts.append((line, toks))
        self.body = None

    # -- declarations
    def _declaration(self, line, toks):
        w = toks[0]
        if w == ("name", "IMPLICIT"):
            return True
        if w == ("name", "INCLUDE"):
            self.includes_mpi = True
            for k in MPI_CONSTS:
                self.decls[k] = Decl(k, I, None, None, False, None, True, None, line)
            return True
        if w == ("name", "DATA"):
            name = toks[1][1]
            vals = [t for t in toks[2:] if t not in (("op", "/"), ("op", ","))]
            consts, sign = [], 1
            for t in vals:
                if t == ("op", "-"):
                    sign = -1
                    continue
                c = literal_value(t[1])
                consts.append(-c if sign < 0 else c)
                sign = 1
            self.data.append((name, consts))
            return True
        if w[0] != "name" or w[1] not in _TYPE_WORDS:
            return False
        if not any(t == ("op", "::") for t in toks) and w[1] != "DOUBLE":
            # "REAL x" without :: (not used by the reference) or a statement
            # that starts with a type word used as a variable
            if len(toks) > 1 and toks[1] == ("op", "="):
                return False
        kind, clen, i = _type_spec(toks)
        attrs, dims, alloc, intent, param = toks[i:], None, False, None, False
        if ("op", "::") in attrs:
            k = attrs.index(("op", "::"))
            attr_toks, ents = attrs[:k], attrs[k + 1:]
        else:
            attr_toks, ents = [], attrs
        for a in _split_top(attr_toks):
            if not a:
                continue
            a0 = a[0][1]
            if a0 == "DIMENSION":
                dims = _dim_spec(a[2:_match_paren(a, 1)], self)
            elif a0 == "ALLOCATABLE":
                alloc = True
            elif a0 == "INTENT":
                intent = "".join(t[1] for t in a[2:-1])
            elif a0 == "PARAMETER":
                param = True
            elif a0 in ("SAVE", "TARGET"):
                pass
            else:
                raise FortranError(f"line {line}: attribute {a0}")
        for ent in _split_top(ents):
            name = ent[0][1]
            edims, init, j = dims, None, 1
            if j < len(ent) and ent[j] == ("op", "("):
                e = _match_paren(ent, j)
                edims = _dim_spec(ent[j + 1:e], self)
                j = e + 1
            if j < len(ent) and ent[j] == ("op", "="):
                init = parse_expr(ent[j + 1:], self)
            self.decls[name] = Decl(name, kind, clen, edims, alloc, intent, param, init, line)
        return True

    def is_array(self, name):
        d = self.decls.get(name)
        return d is not None and d.dims is not None

    # -- expression building blocks
    def variable(self, name):
        d = self.decls.get(name)
        if d is None:
            raise FortranError(f"{self.name}: undeclared {name}")
        if d.dims is not None:
            return lambda fr: fr.v[name].a
        return lambda fr: fr.v[name]

    def designator_or_call(self, name, args):
        if self.is_array(name):
            subs = [a for a in args]
            if all(a[0] == "e" for a in subs):
                fs = [a[1] for a in subs]
                if len(fs) == 1:
                    f0, = fs
                    return lambda fr: _elem1(fr.v[name], f0(fr), name)
                if len(fs) == 3:
                    f0, f1, f2 = fs
                    return lambda fr: _elem3(fr.v[name], f0(fr), f1(fr), f2(fr), name,
                                             fr.interp.linear)
                return lambda fr: (lambda A: A.a[_idx(A, [f(fr) for f in fs], name)])(fr.v[name])
            sec = self._section(subs)
            return lambda fr: (lambda A: A.a[_slices(A, sec(fr), name)])(fr.v[name])
        if name in self.interp.intrinsics:
            fn = self.interp.intrinsics[name]
            pos = [a[1] for a in args if a[0] == "e"]
            kws = {a[1]: a[2] for a in args if a[0] == "kw"}
            if any(a[0] == "s" for a in args):
                raise FortranError(f"section as an argument of {name}")
            if name == "REAL" and "KIND" in kws:
                kf = kws["KIND"]
                return lambda fr: fn(pos[0](fr), kf(fr))
            if len(pos) == 1:
                p0, = pos
                return lambda fr: fn(p0(fr))
            if len(pos) == 2:
                p0, p1 = pos
                return lambda fr: fn(p0(fr), p1(fr))
            return lambda fr: fn(*[p(fr) for p in pos])
        raise FortranError(f"{self.name}: {name}(...) is neither an array nor a known function")

    def _section(self, subs):
        parts = []
        for a in subs:
            if a[0] == "e":
                parts.append(a[1])
            else:
                lo, hi, st = a[1:]
                parts.append((lo, hi, st))

        def ev(fr):
            out = []
            for p in parts:
                if isinstance(p, tuple):
                    out.append(tuple(None if q is None else q(fr) for q in p))
                else:
                    out.append(p(fr))
            return out

        return ev

    def ref(self, toks):
        """An argument or assignment target: a _Ref."""
        if toks and toks[0][0] == "name" and (len(toks) == 1 or (
                toks[1] == ("op", "(") and _match_paren(toks, 1) == len(toks) - 1)):
            name = toks[0][1]
            d = self.decls.get(name)
            if d is not None and len(toks) == 1:
                if d.dims is not None:
                    return _Ref(lambda fr: fr.v[name].a, lambda fr: fr.v[name].a, None)
                kind = d.kind

                def setv(fr, v, name=name, kind=kind, d=d):
                    fr.v[name] = _store_scalar(v, kind, d.clen)

                return _Ref(lambda fr: fr.v[name], None, setv)
            if d is not None and d.dims is not None:
                p = _Parser(toks[2:], self)
                args = p.arglist()
                sec = self._section(args)

                def view(fr, name=name, sec=sec):
                    A = fr.v[name]
                    s = _slices(A, sec(fr), name)
                    if all(isinstance(x, int) for x in s):  # element: a 1-element view
                        s = tuple(slice(x, x + 1) for x in s)
                        return A.a[s].reshape(())
                    return A.a[s]

                def setv(fr, v, view=view):
                    view(fr)[...] = v

                return _Ref(lambda fr: _value_of(view(fr)), view, setv)
        e = parse_expr(toks, self)
        return _Ref(e, None, None)


def _value_of(v):
    if isinstance(v, np.ndarray) and v.ndim == 0:
        return v[()]
    return v


def _elem1(A, i, name):
    j = i - A.lb[0]
    if j < 0 or j >= A.a.shape[0]:
        raise FortranError(f"{name}: subscript {i} outside {A.lb[0]}:{A.lb[0] + A.a.shape[0] - 1}")
    return A.a[j]


def _elem3(A, i, j, k, name, linear=False):
    a = A.a
    lb = A.lb
    i0, j0, k0 = i - lb[0], j - lb[1], k - lb[2]
    s = a.shape
    if not (0 <= i0 < s[0] and 0 <= j0 < s[1] and 0 <= k0 < s[2]):
        if not linear:
            raise FortranError(f"{name}({i},{j},{k}) outside its bounds")
        return _flat(A, name)[_linear_offset(A, (i0, j0, k0), name)]
    return a[i0, j0, k0]


def _linear_offset(A, idx0, name):
    """Column-major offset of the 0-based subscripts idx0 in A's storage, as
    code compiled without bounds checks addresses an element whose
    subscript leaves its dimension; FortranError when it leaves the storage."""
    off, stride = 0, 1
    for d, i in enumerate(idx0):
        off += i * stride
        stride *= A.a.shape[d]
    if not 0 <= off < A.a.size:
        raise FortranError(f"{name}: element outside the array's storage")
    return off


def _flat(A, name):
    if not A.a.flags.f_contiguous:
        raise FortranError(f"{name}: linear addressing of a non-contiguous array")
    return A.a.reshape(-1, order="F")


def _store_scalar(v, kind, clen):
    if kind == CH:
        s = str(v)
        return s[:clen].ljust(clen) if clen else s
    if isinstance(v, np.ndarray):
        raise FortranError("array assigned to a scalar")
    return convert(v, kind)


# ------------------------------------------------------------- statements
_SIG_EXIT, _SIG_RETURN = "EXIT", "RETURN"  # CYCLE ends the body like a normal pass


class _Builder:
    """Builds the executable tree of a unit from (line, tokens) statements."""

    def __init__(self, unit, stmts):
        self.u, self.s, self.i = unit, stmts, 0

    def block(self, ends):
        nodes = []
        while self.i < len(self.s):
            line, toks = self.s[self.i]
            head = _head(toks)
            if head in ends:
                return nodes, head
            self.i += 1
            nodes.append((line, self.stmt(line, toks, head)))
        if ends:
            raise FortranError(f"{self.u.name}: missing {ends}")
        return nodes, None

    def stmt(self, line, toks, head):
        u = self.u
        if head == "DO":
            return self.do(line, toks)
        if head == "IF":
            j = _match_paren(toks, 1)
            cond = parse_expr(toks[2:j], u)
            rest = toks[j + 1:]
            if rest == [("name", "THEN")]:
                return self.if_block(cond)
            inner = self.stmt(line, rest, _head(rest))
            return lambda fr: inner(fr) if _truth(cond(fr)) else None
        if head == "WHERE":
            j = _match_paren(toks, 1)
            mask = parse_expr(toks[2:j], u)
            rest = toks[j + 1:]
            if rest:
                return _where(mask, [self.where_assign(line, rest)], [])
            body, other = [], []
            cur = body
            while True:
                if self.i >= len(self.s):
                    raise FortranError(f"line {line}: WHERE without END WHERE")
                ln, t = self.s[self.i]
                self.i += 1
                h = _head(t)
                if h == "ELSEWHERE":
                    cur = other
                elif h == "ENDWHERE":
                    return _where(mask, body, other)
                else:
                    cur.append(self.where_assign(ln, t))
        if head == "SELECT":
            j = _match_paren(toks, 2)
            sel = parse_expr(toks[3:j], u)
            cases, default = [], None
            _, h = self.block(("CASE", "ENDSELECT"))
            while h == "CASE":
                ctoks = self.s[self.i][1]
                self.i += 1
                body, h = self.block(("CASE", "ENDSELECT"))
                if ctoks[1] == ("name", "DEFAULT"):
                    default = body
                else:
                    k = _match_paren(ctoks, 1)
                    vals = [parse_expr(p, u) for p in _split_top(ctoks[2:k])]
                    cases.append((vals, body))
            self.i += 1

            def select(fr):
                v = sel(fr)
                for vals, body in cases:
                    if any(relation("==", v, f(fr)) for f in vals):
                        return _run(body, fr)
                if default is not None:
                    return _run(default, fr)
                return None

            return select
        if head == "CALL":
            return self.call(toks)
        if head in ("EXIT", "CYCLE", "RETURN"):
            sig = head
            return lambda fr: sig
        if head == "STOP":
            def stop(fr):
                raise Stop("STOP")
            return stop
        if head == "ALLOCATE":
            return self.allocate(toks)
        if head == "DEALLOCATE":
            names = [p[0][1] for p in _split_top(toks[2:_match_paren(toks, 1)])]

            def dealloc(fr):
                for n in names:
                    fr.v[n] = None

            return dealloc
        if head in ("OPEN", "CLOSE", "READ", "WRITE", "PRINT"):
            return self.io(head, toks)
        if head == "ASSIGN":
            return self.assign(toks)
        raise FortranError(f"{u.name} line {line}: unsupported statement {' '.join(str(t[1]) for t in toks)}")

    def where_assign(self, line, toks):
        """An assignment inside WHERE: (target _Ref, rhs closure)."""
        k = _assign_split(toks)
        if k is None or _head(toks) != "ASSIGN":
            raise FortranError(f"line {line}: only assignments inside WHERE")
        return self.u.ref(toks[:k]), parse_expr(toks[k + 1:], self.u)

    def if_block(self, cond):
        branches = []
        body, h = self.block(("ELSEIF", "ELSE", "ENDIF"))
        branches.append((cond, body))
        while h == "ELSEIF":
            toks = self.s[self.i][1]
            self.i += 1
            k = 1 if toks[0] == ("name", "ELSEIF") else 2
            j = _match_paren(toks, k)
            c = parse_expr(toks[k + 1:j], self.u)
            body, h = self.block(("ELSEIF", "ELSE", "ENDIF"))
            branches.append((c, body))
        other = None
        if h == "ELSE":
            self.i += 1
            other, h = self.block(("ENDIF",))
        self.i += 1

        def run_if(fr):
            for c, b in branches:
                if _truth(c(fr)):
                    return _run(b, fr)
            if other is not None:
                return _run(other, fr)
            return None

        return run_if

    def do(self, line, toks):
        if len(toks) > 1 and toks[1] == ("name", "WHILE"):
            j = _match_paren(toks, 2)
            cond = parse_expr(toks[3:j], self.u)
            body, _ = self.block(("ENDDO",))
            self.i += 1

            def run_while(fr):
                while _truth(cond(fr)):
                    s = _run(body, fr)
                    if s == _SIG_EXIT:
                        break
                    if s == _SIG_RETURN:
                        return s
                return None

            return run_while
        var = toks[1][1]
        parts = _split_top(toks[3:])
        lo, hi = parse_expr(parts[0], self.u), parse_expr(parts[1], self.u)
        st = parse_expr(parts[2], self.u) if len(parts) > 2 else (lambda fr: 1)
        body, _ = self.block(("ENDDO",))
        self.i += 1

        def run_do(fr):
            a, b, c = lo(fr), hi(fr), st(fr)
            n = max(_int_div(b - a + c, c), 0)
            v = a
            for _ in range(n):
                fr.v[var] = v
                s = _run(body, fr)
                if s == _SIG_EXIT:
                    return None
                if s == _SIG_RETURN:
                    return s
                v += c
            fr.v[var] = v
            return None

        return run_do

    def call(self, toks):
        name = toks[1][1]
        args = []
        if len(toks) > 2:
            j = _match_paren(toks, 2)
            args = [self.u.ref(p) for p in _split_top(toks[3:j]) if p]
        interp = self.u.interp
        unit = self.u

        def run_call(fr):
            hook = interp.call_hooks.get(name) or _MPI.get(name)
            if hook is not None:
                hook(fr, args)
                return None
            callee = interp.unit(unit.path, name)
            interp.invoke(callee, args, fr)
            return None

        return run_call

    def allocate(self, toks):
        items = []
        for p in _split_top(toks[2:_match_paren(toks, 1)]):
            name = p[0][1]
            dims = _dim_spec(p[2:_match_paren(p, 1)], self.u)
            items.append((name, dims))
        unit = self.u

        def run_alloc(fr):
            for name, dims in items:
                shape, lb = _eval_dims(dims, fr)
                kind = unit.decls[name].kind
                fr.v[name] = FArr(np.zeros(shape, dtype=_NP[kind], order="F"), lb, kind)
            return None

        return run_alloc

    def io(self, head, toks):
        interp, u = self.u.interp, self.u
        if head == "PRINT":
            return lambda fr: None
        j = _match_paren(toks, 1)
        ctl = _split_top(toks[2:j])
        rest = toks[j + 1:]
        kw = {}
        pos = []
        for c in ctl:
            if len(c) > 1 and c[0][0] == "name" and c[1] == ("op", "="):
                kw[c[0][1]] = c[2:]
            else:
                pos.append(c)
        unit_toks = kw.get("UNIT", pos[0] if pos else None)
        if head == "OPEN":
            ue, fe = parse_expr(unit_toks, u), parse_expr(kw["FILE"], u)

            def run_open(fr):
                interp.files[ue(fr)] = fe(fr).strip()
                return None

            return run_open
        if head == "CLOSE":
            ue = parse_expr(unit_toks, u)

            def run_close(fr):
                interp.files.pop(ue(fr), None)
                return None

            return run_close
        items = [p for p in _split_top(rest) if p]
        if head == "READ":
            ue = parse_expr(unit_toks, u)
            refs = [u.ref(p) for p in items]

            def run_read(fr):
                key = ue(fr)
                fname = interp.files.get(key, str(key))
                for r in refs:
                    target = r.view(fr) if r.view else None
                    if target is None:
                        raise FortranError("READ into a scalar is not supported")
                    val = interp.on_read(fname, target.shape, target.dtype)
                    target[...] = np.asarray(val).astype(target.dtype)
                return None

            return run_read
        # WRITE: internal (to a CHARACTER variable) or external
        ut = unit_toks
        internal = len(ut) == 1 and ut[0][0] == "name" and u.decls.get(ut[0][1]) is not None \
            and u.decls[ut[0][1]].kind == CH
        vals = [parse_expr(p, u) for p in items]
        if internal:
            target = u.ref(ut)
            fmt = pos[1] if len(pos) > 1 else kw.get("FMT")
            fmt_s = fmt[0][1] if fmt and fmt[0][0] == "str" else None
            m = re.fullmatch(r"\(\s*I(\d+)\s*\)", fmt_s or "", re.I)
            if not m:
                raise FortranError(f"internal WRITE format {fmt_s!r}")
            width = int(m.group(1))

            def run_iwrite(fr):
                s = str(vals[0](fr)).rjust(width)
                target.set(fr, "*" * width if len(s) > width else s)
                return None

            return run_iwrite
        ue = parse_expr(ut, u)

        def run_write(fr):
            key = ue(fr)
            interp.on_write(interp.files.get(key, str(key)), [v(fr) for v in vals])
            return None

        return run_write

    def assign(self, toks):
        k = _assign_split(toks)
        lhs, rhs_t = toks[:k], toks[k + 1:]
        rhs = parse_expr(rhs_t, self.u)
        name = lhs[0][1]
        d = self.u.decls.get(name)
        if d is None:
            raise FortranError(f"{self.u.name}: assignment to undeclared {name}")
        if len(lhs) == 1 and d.dims is None:
            kind, clen = d.kind, d.clen

            def set_scalar(fr):
                v = _store_scalar(rhs(fr), kind, clen)
                o = fr.ovr
                if o and name in o:
                    v = o[name]
                fr.v[name] = v
                return None

            return set_scalar
        if len(lhs) == 1:
            def set_whole(fr):
                A = fr.v[name]
                v = rhs(fr)
                if isinstance(v, np.ndarray):
                    v = np.array(v, copy=True)
                A.a[...] = convert(v, A.kind) if kind_of(v) != A.kind else v
                return None

            return set_whole
        p = _Parser(lhs[2:], self.u)
        args = p.arglist()
        if all(a[0] == "e" for a in args) and len(args) == 3:
            f0, f1, f2 = (a[1] for a in args)

            def set_elem3(fr):
                A = fr.v[name]
                v = rhs(fr)
                i, j, kk = f0(fr) - A.lb[0], f1(fr) - A.lb[1], f2(fr) - A.lb[2]
                s = A.a.shape
                if not (0 <= i < s[0] and 0 <= j < s[1] and 0 <= kk < s[2]):
                    if not fr.interp.linear:
                        raise FortranError(f"{name}: store outside its bounds")
                    _flat(A, name)[_linear_offset(A, (i, j, kk), name)] = convert(v, A.kind)
                    return None
                A.a[i, j, kk] = convert(v, A.kind)
                return None

            return set_elem3
        sec = self.u._section(args)

        def set_section(fr):
            A = fr.v[name]
            v = rhs(fr)
            if isinstance(v, np.ndarray):
                v = np.array(v, copy=True)
            tgt = _slices(A, sec(fr), name)
            A.a[tgt] = convert(v, A.kind) if kind_of(v) != A.kind else v
            return None

        return set_section


def _eval_dims(dims, fr):
    shape, lb = [], []
    for d in dims:
        if d is None:
            raise FortranError("deferred shape outside ALLOCATE")
        lo, hi = d[0](fr), d[1](fr)
        shape.append(max(hi - lo + 1, 0))
        lb.append(lo)
    return tuple(shape), tuple(lb)


def _truth(v):
    if isinstance(v, np.ndarray):
        raise FortranError("array condition in IF / DO WHILE")
    return bool(v)


def _run(nodes, fr):
    hooks = fr.interp.line_hooks
    for line, n in nodes:
        if hooks and line in hooks:
            pre, post = hooks[line]
            if pre:
                pre(fr)
            s = n(fr)
            if post:
                post(fr)
        else:
            s = n(fr)
        if s is not None:
            return s
    return None


def _where(mask, body, other):
    def run_where(fr):
        m = mask(fr)
        if not isinstance(m, np.ndarray):
            raise FortranError("WHERE with a scalar mask")
        for sel, items in ((m, body), (np.logical_not(m), other)):
            for tgt, rhs in items:
                view = tgt.view(fr)
                v = rhs(fr)
                if view.shape != sel.shape:
                    raise FortranError("WHERE target does not conform with the mask")
                if isinstance(v, np.ndarray):
                    view[sel] = convert(v, kind_of(view))[sel]
                else:
                    view[sel] = convert(v, kind_of(view))
        return None

    return run_where


def _head(toks):
    """The statement keyword (ASSIGN for assignments)."""
    if not toks:
        return None
    t0 = toks[0]
    if t0[0] != "name":
        raise FortranError(f"statement starting with {t0}")
    w = t0[1]
    nxt = toks[1] if len(toks) > 1 else None
    if nxt == ("op", "=") or (nxt == ("op", "(") and _assign_split(toks) is not None
                              and w not in ("IF", "WHERE", "CALL", "READ", "WRITE", "OPEN", "CLOSE",
                                            "ALLOCATE", "DEALLOCATE", "SELECT", "CASE", "ELSEIF")):
        return "ASSIGN"
    two = w + (toks[1][1] if nxt and nxt[0] == "name" else "")
    if two in ("ENDDO", "ENDIF", "ENDWHERE", "ENDSELECT", "ELSEIF", "ELSEWHERE", "ENDPROGRAM",
               "ENDSUBROUTINE"):
        return two
    if w in ("ENDDO", "ENDIF", "ENDWHERE", "ELSEIF", "ELSEWHERE", "ENDSELECT"):
        return w
    if w == "SELECT":
        return "SELECT"
    return w


def _assign_split(toks):
    depth = 0
    for k, t in enumerate(toks):
        if t == ("op", "("):
            depth += 1
        elif t == ("op", ")"):
            depth -= 1
        elif depth == 0 and t == ("op", "="):
            return k
    return None


# -------------------------------------------------------------------- MPI
def _mpi_set(ref, fr, v):
    if ref.set is None:
        raise FortranError("MPI output argument is not a variable")
    ref.set(fr, v)


def _mpi_allgather(fr, a):
    view = a[3].view(fr)
    if view is None:
        raise FortranError("MPI_ALLGATHER receive buffer is not an array")
    flat = view.reshape(-1)
    flat[0] = a[0].get(fr)
    _mpi_set(a[7], fr, 0)


_MPI = {
    "MPI_INIT": lambda fr, a: _mpi_set(a[0], fr, 0),
    "MPI_COMM_RANK": lambda fr, a: (_mpi_set(a[1], fr, 0), _mpi_set(a[2], fr, 0)),
    "MPI_COMM_SIZE": lambda fr, a: (_mpi_set(a[1], fr, 1), _mpi_set(a[2], fr, 0)),
    "MPI_ALLGATHER": _mpi_allgather,
    "MPI_BARRIER": lambda fr, a: _mpi_set(a[1], fr, 0),
    "MPI_FINALIZE": lambda fr, a: _mpi_set(a[0], fr, 0),
}


# ------------------------------------------------------------------ driver
class Interp:
    """Parses Fortran source files and runs their units.

    overrides: {unit name: {variable: value}} -- a PARAMETER takes the value
    instead of its initialiser, a scalar variable takes it after every
    assignment to it (how a fixed production size is replaced by a small
    one).  Hooks: on_read(file, shape, dtype) -> data, on_write(file, values),
    call_hooks {name: f(frame, refs)} for CALLs, line_hooks {line: (before,
    after)} on the statements starting at a line.  sum_order "sequential"
    (the compiled reference's) or "planes" (the C oracle's, see _sum_planes).
    bounds "check" (a subscript outside its dimension raises) or "linear"
    (an element of a rank-3 array whose subscript leaves its dimension is
    addressed by its column-major offset, as compiled code without bounds
    checks does, as long as that stays inside the array's storage).
    """

    def __init__(self, paths, overrides=None, sum_order="sequential", bounds="check"):
        if bounds not in ("check", "linear"):
            raise ValueError(f"bounds {bounds!r}")
        self.linear = bounds == "linear"
        self.overrides = {k.upper(): {n.upper(): v for n, v in d.items()}
                          for k, d in (overrides or {}).items()}
        self.intrinsics = dict(INTRINSICS)
        if sum_order == "planes":
            self.intrinsics["SUM"] = _sum_planes
        elif sum_order != "sequential":
            raise ValueError(f"sum_order {sum_order!r}")
        self.units: dict[tuple[str, str], Unit] = {}
        self.files = {}
        self.call_hooks = {}
        self.line_hooks = {}
        self.on_read = self._no_read
        self.on_write = lambda fname, values: None
        for path in paths:
            self._load(str(path))

    @staticmethod
    def _no_read(fname, shape, dtype):
        raise FortranError(f"READ from {fname} without a hook")

    def _load(self, path):
        text = open(path).read()
        cur, stmts = None, []
        for line, s in logical_lines(text):
            toks = tokenize(s)
            w = toks[0][1] if toks and toks[0][0] == "name" else None
            if cur is None:
                if w in ("PROGRAM", "SUBROUTINE"):
                    name = toks[1][1]
                    args = []
                    if w == "SUBROUTINE" and len(toks) > 2 and toks[2] == ("op", "("):
                        args = [t[1] for t in toks[3:_match_paren(toks, 2)] if t[0] == "name"]
                    cur, stmts = (name, w, args, line), []
                    continue
                raise FortranError(f"{path}:{line}: statement outside a program unit")
            if w == "END" and (len(toks) == 1 or toks[1][1] in ("PROGRAM", "SUBROUTINE")) \
                    or w in ("ENDPROGRAM", "ENDSUBROUTINE"):
                name, kind, args, first = cur
                u = Unit(name, kind, args, stmts, self, path)
                u.first_line, u.last_line = first, line
                b = _Builder(u, u.stmts)
                u.body, _ = b.block(())
                self.units[(path, name)] = u
                cur = None
                continue
            stmts.append((line, toks))
        if cur is not None:
            raise FortranError(f"{path}: unit {cur[0]} has no END")

    def unit(self, path, name):
        u = self.units.get((str(path), name.upper()))
        if u is None:
            raise FortranError(f"no unit {name} in {path}")
        return u

    # -- frames
    def _frame(self, u, bind=None):
        fr = Frame(u, self)
        bind = bind or {}
        fr.v.update(bind)
        ovr = fr.ovr
        static = u.kind == "PROGRAM"
        for name, d in u.decls.items():
            if name in bind:
                continue
            if d.param:
                if name in MPI_CONSTS:
                    fr.v[name] = MPI_CONSTS[name]
                else:
                    fr.v[name] = ovr[name] if name in ovr else _store_scalar(d.init(fr), d.kind, d.clen)
            elif d.dims is not None:
                if d.alloc or any(x is None for x in d.dims):
                    fr.v[name] = None
                else:
                    shape, lb = _eval_dims(d.dims, fr)
                    fill = 0 if static or d.kind not in (R4, R8) else np.nan
                    fr.v[name] = FArr(np.full(shape, fill, dtype=_NP[d.kind], order="F"), lb, d.kind)
            else:
                if d.kind == CH:
                    fr.v[name] = " " * (d.clen or 0)
                elif d.kind in (R4, R8):
                    fr.v[name] = convert(0 if static else np.nan, d.kind)
                elif d.kind == L:
                    fr.v[name] = False
                else:
                    fr.v[name] = 0
                if d.init is not None:
                    fr.v[name] = _store_scalar(d.init(fr), d.kind, d.clen)
        for name, consts in u.data:
            A = fr.v[name]
            vals = np.array([convert(c, A.kind) for c in consts], dtype=_NP[A.kind])
            A.a.reshape(-1, order="F")[...] = vals  # a fresh F-ordered array: reshape is a view
        return fr

    def invoke(self, u, refs, caller):
        if len(refs) != len(u.args):
            raise FortranError(f"{u.name}: {len(refs)} arguments for {len(u.args)} dummies")
        fr = Frame(u, self)
        pairs = list(zip(u.args, refs))
        for dn, r in pairs:  # scalars first: the explicit shapes use them
            d = u.decls[dn]
            if d.dims is None:
                fr.v[dn] = _store_scalar(r.get(caller), d.kind, d.clen)
        for dn, r in pairs:
            d = u.decls[dn]
            if d.dims is None:
                continue
            shape, lb = _eval_dims(d.dims, fr)  # explicit shape from the scalar dummies
            view = r.view(caller) if r.view else None
            if view is None:
                view = np.asarray(r.get(caller))
            if kind_of(view) != d.kind:
                raise FortranError(f"{u.name}: argument {dn} of kind {kind_of(view)}, dummy {d.kind}")
            n = int(np.prod(shape))
            flat = np.asarray(view).reshape(-1, order="F")
            if flat.size < n:
                raise FortranError(f"{u.name}: actual {dn} has {flat.size} elements, dummy {n}")
            data = np.array(flat[:n], dtype=_NP[d.kind]).reshape(shape, order="F")
            fr.v[dn] = FArr(data, lb, d.kind)
        full = self._frame(u, bind=dict(fr.v))
        _run(u.body, full)
        for dn, r in pairs:
            d = u.decls[dn]
            if d.intent == "IN":
                continue
            if d.dims is None:
                if r.set is not None:
                    r.set(caller, full.v[dn])
                continue
            view = r.view(caller) if r.view else None
            if view is None:
                continue
            data = full.v[dn].a.reshape(-1, order="F")
            if view.size == data.size:
                view[...] = data.reshape(view.shape, order="F")
            else:
                tmp = np.array(view).reshape(-1, order="F")
                tmp[:data.size] = data
                view[...] = tmp.reshape(view.shape, order="F")

    def call(self, path, name, *args):
        """Run a SUBROUTINE on Python values; arrays are updated in place
        unless the dummy is INTENT(IN).  Arguments: ints, floats,
        numpy.float32 or numpy arrays (whose element kind must match)."""
        u = self.unit(path, name)
        holders = []
        refs = []
        for a in args:
            if isinstance(a, np.ndarray):
                refs.append(_Ref(lambda fr, a=a: a, lambda fr, a=a: a, None))
            else:
                box = [a]
                holders.append(box)
                refs.append(_Ref(lambda fr, box=box: box[0], None,
                                 lambda fr, v, box=box: box.__setitem__(0, v)))
        caller = Frame(u, self)
        self.invoke(u, refs, caller)
        return [b[0] for b in holders]

    def run_program(self, path, name):
        """Run a main program until it ends or a hook raises Stop; returns its frame."""
        u = self.unit(path, name)
        fr = self._frame(u)
        try:
            _run(u.body, fr)
        except Stop:
            pass
        return fr

    def exec_lines(self, path, name, first, last, preset):
        """Run the statements of a unit that start on lines first..last (a
        sequence of whole statements and blocks) in a new frame of the unit,
        after setting the variables in preset (arrays as FArr or numpy arrays
        of the declared shape); returns the frame."""
        u = self.unit(path, name)
        sub = [(ln, t) for ln, t in u.stmts if first <= ln <= last]
        nodes, h = _Builder(u, sub).block(())
        fr = self._frame(u)
        for k, v in preset.items():
            k = k.upper()
            cur = fr.v.get(k)
            if isinstance(cur, FArr):
                if tuple(np.shape(v)) != cur.a.shape:
                    raise FortranError(f"preset {k}: shape {np.shape(v)} for {cur.a.shape}")
                cur.a[...] = np.asarray(v).astype(cur.a.dtype)
            else:
                fr.v[k] = _store_scalar(v, u.decls[k].kind, u.decls[k].clen)
        try:
            _run(nodes, fr)
        except Stop:
            pass
        return fr

    def line_of(self, path, pattern, start=1):
        """The first line at or after start whose text matches pattern (re)."""
        rx = re.compile(pattern, re.I)
        for no, raw in enumerate(open(path).read().splitlines(), 1):
            if no >= start and rx.search(_strip_comment(raw)):
                return no
        raise FortranError(f"{path}: no line matches {pattern!r}")
