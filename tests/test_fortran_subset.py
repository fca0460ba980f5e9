"""The Fortran-subset interpreter that produces the reference vectors.  CPU only.

Its semantics are checked here on small programs of this file's own, against
values computed independently; the last test re-runs the quick cases of
tests/golden/make_reference_golden.py on the reference's sources, when they
are present, and compares them with the committed fixture.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import fortran_subset as fs  # noqa: E402

f32 = np.float32


def run(tmp_path, src, name="T", **kw):
    p = tmp_path / "t.f90"
    p.write_text(src)
    it = fs.Interp([p], **kw)
    return it, p, it.run_program(p, name).v


def test_literal_kinds_and_promotion(tmp_path):
    _, _, v = run(tmp_path, """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8) :: a, b, c, d, e
REAL(KIND=4) :: s
INTEGER :: i, j, m
a = 0.1
b = 0.1d0
c = 1.05625e-02 *0.125 *0.75
s = 3.25**2
i = 7/2
j = -7/2
m = MOD(-7,3)
d = 2*0.5d0
e = -7.02 -0.83d3*b +0.05*(1.0d3*b)**2
END PROGRAM T
""")
    assert v["A"] == float(f32(0.1)) and v["B"] == 0.1
    assert v["C"] == float(f32(f32(f32(0.0105625) * f32(0.125)) * f32(0.75)))
    assert isinstance(v["S"], f32) and v["S"] == 10.5625
    assert (v["I"], v["J"], v["M"]) == (3, -3, -1)
    q = 1.0e3 * 0.1
    assert v["E"] == (float(f32(-7.02)) - 0.83e3 * 0.1) + float(f32(0.05)) * (q * q)


def test_binary32_literal_is_rounded_once():
    # just above the midpoint between 1 and its binary32 successor: rounding
    # to binary64 first lands on the midpoint and then ties to even (1.0)
    assert fs.f32_from_text("1.000000059604644775390625001") == f32(1.0 + 2.0 ** -23)
    assert fs.f32_from_text("1.000000059604644775390625") == f32(1.0)  # the tie itself
    assert fs.f32_from_text("0.0312") == f32(0.0312)


def test_integer_powers_and_transcendentals(tmp_path):
    _, _, v = run(tmp_path, """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8) :: x, p2, p3, p5, pr, ex, th
REAL(KIND=4) :: xs, es
x = 1.1d0
p2 = x**2
p3 = x**3
p5 = x**5
pr = x**2.5d0
ex = EXP(x)
th = TANH(x)
xs = 1.1
es = EXP(xs)
END PROGRAM T
""")
    x = 1.1
    assert v["P2"] == x * x and v["P3"] == x * (x * x)
    x2 = x * x
    assert v["P5"] == x * (x2 * x2)  # libgcc __powidf2: y = x; x = x^2; x = x^4; y = y*x^4
    assert v["PR"] == math.pow(x, 2.5) and v["EX"] == math.exp(x) and v["TH"] == math.tanh(x)
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    libm.expf.restype, libm.expf.argtypes = ctypes.c_float, [ctypes.c_float]
    assert v["ES"] == f32(libm.expf(float(f32(1.1))))


def test_sum_is_sequential_in_column_major_order(tmp_path):
    _, _, v = run(tmp_path, """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8), DIMENSION(2,2) :: a
REAL(KIND=8), DIMENSION(4) :: b
REAL(KIND=8) :: s1, s2
a(1,1) = 1.0d16
a(2,1) = 1.0d0
a(1,2) = -1.0d16
a(2,2) = 1.0d0
b(1) = 1.0d16
b(2) = -1.0d16
b(3) = 1.0d0
b(4) = 1.0d0
s1 = SUM(a)
s2 = SUM(b)
END PROGRAM T
""")
    # column-major sequence 1e16, 1, -1e16, 1: the first 1 is absorbed
    assert v["S1"] == 1.0
    assert v["S2"] == 2.0


def test_planes_order_sums_each_z_plane_first(tmp_path):
    src = """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8), DIMENSION(1,2,2) :: a
REAL(KIND=8) :: s
a(1,1,1) = 1.0d16
a(1,2,1) = 1.0d0
a(1,1,2) = -1.0d16
a(1,2,2) = 1.0d0
s = SUM(a)
END PROGRAM T
"""
    _, _, seq = run(tmp_path, src)
    _, _, pl = run(tmp_path, src, sum_order="planes")
    assert seq["S"] == 1.0  # ((1e16 + 1) - 1e16) + 1
    assert pl["S"] == 0.0   # (1e16 + 1) + (-1e16 + 1)


def test_loops_where_select_and_internal_write(tmp_path):
    _, _, v = run(tmp_path, """
PROGRAM T
IMPLICIT NONE
INTEGER :: i, k, n, z
REAL(KIND=8), DIMENSION(0:3) :: a, b
CHARACTER(LEN=4) :: s
k = 0
DO i = 1, 10
  IF ( i == 4 ) CYCLE
  k = k + i
  IF ( k > 20 ) EXIT
ENDDO
z = 0
DO n = 5, 1
  z = z + 1
ENDDO
a(0) = 1.0
a(1) = -2.0
a(2) = 3.0
a(3) = -4.0
WHERE ( a > 0.0 )
  a = -a
  b = a
ELSEWHERE
  b = 7.0
END WHERE
SELECT CASE (k)
  CASE (24)
    z = z + 100
  CASE (1)
    z = -1
END SELECT
WRITE(s,"(I4)") 1000+k
END PROGRAM T
""")
    assert (v["I"], v["K"]) == (7, 24)        # EXIT keeps the current value
    assert v["N"] == 5 and v["Z"] == 100      # zero-trip loop: n = 5, z untouched
    assert list(v["A"].a) == [-1.0, -2.0, -3.0, -4.0]
    assert list(v["B"].a) == [-1.0, 7.0, -3.0, 7.0]  # mask taken once, new a seen
    assert v["S"] == "1024"


def test_data_sign_and_floor(tmp_path):
    _, _, v = run(tmp_path, """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8), DIMENSION(0:2) :: t
REAL(KIND=8) :: a, b, c
INTEGER :: f1, f2
DATA t / 0, 6.3826e+00, -1.5d0 /
a = DSIGN(2.0d0, -0.0d0)
b = DSIGN(-3.0d0, 1.0d0)
c = MAX(1, 2.5, 0.5d0)
f1 = FLOOR(-0.5d0)
f2 = FLOOR(2.999d0)
END PROGRAM T
""")
    assert list(v["T"].a) == [0.0, float(f32(6.3826)), -1.5]  # REAL(4) literal widened
    assert v["A"] == -2.0 and math.copysign(1.0, v["A"]) < 0 and v["B"] == 3.0
    assert v["C"] == 2.5 and (v["F1"], v["F2"]) == (-1, 2)


def test_ieee_results_where_python_raises():
    f = fs.INTRINSICS
    assert f["LOG"](0.0) == -math.inf and math.isnan(f["LOG"](-1.0))
    assert f["EXP"](1000.0) == math.inf and f["EXP"](-1000.0) == 0.0
    assert math.isnan(f["SQRT"](-1.0))


def test_out_of_bounds_access_raises(tmp_path):
    p = tmp_path / "t.f90"
    p.write_text("""
PROGRAM T
IMPLICIT NONE
REAL(KIND=8), DIMENSION(3) :: a
INTEGER :: i
DO i = 1, 4
  a(i) = 1.0
ENDDO
END PROGRAM T
""")
    it = fs.Interp([p])
    with pytest.raises(fs.FortranError):
        it.run_program(p, "T")


def test_sequence_association_and_storage(tmp_path):
    _, _, v = run(tmp_path, """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8), DIMENSION(3,4) :: a
REAL(KIND=8), ALLOCATABLE :: c(:)
INTEGER :: i, j
DO j = 1, 4
  DO i = 1, 3
    a(i,j) = 10*i + j
  ENDDO
ENDDO
CALL twice(4, a(2:3,1:2))
ALLOCATE(c(0:2))
END PROGRAM T
SUBROUTINE twice(n, x)
IMPLICIT NONE
INTEGER, INTENT(IN) :: n
REAL(KIND=8), INTENT(INOUT), DIMENSION(n) :: x
REAL(KIND=8), DIMENSION(2) :: w
x(1:n) = 2*x(1:n)
END SUBROUTINE twice
""")
    a = v["A"].a
    # the section a(2:3,1:2) is the sequence 21, 31, 22, 32 in the dummy
    assert a[1, 0] == 42 and a[2, 0] == 62 and a[1, 1] == 44 and a[2, 1] == 64
    assert a[0, 0] == 11 and a[1, 2] == 23  # elements outside the section untouched
    assert v["C"].lb == (0,) and np.all(v["C"].a == 0)


def test_automatic_arrays_start_undefined(tmp_path):
    p = tmp_path / "t.f90"
    p.write_text("""
SUBROUTINE s(n, y)
IMPLICIT NONE
INTEGER, INTENT(IN) :: n
REAL(KIND=8), INTENT(OUT), DIMENSION(n) :: y
REAL(KIND=8), DIMENSION(n) :: w
y(1:n) = w(1:n)
END SUBROUTINE s
""")
    it = fs.Interp([p])
    y = np.zeros(3)
    it.call(p, "s", 3, y)
    assert np.isnan(y).all()


def _reference_src():
    import make_reference_golden as M
    src = Path(M.DEFAULT_REFERENCE) / "src" / "frtrn"
    return M, src


def test_fixture_reproduces_from_the_reference_sources():
    M, src = _reference_src()
    if not src.is_dir():
        pytest.skip("the reference's sources are not on this machine")
    G = np.load(GOLDEN / "reference_v1.npz")
    out = {}
    for case in (M.case_tbl, M.case_dmn, M.case_cmbn, M.case_sbmes, M.case_sbmes_planes):
        case(src, out)
    for k, a in out.items():
        assert k in G.files, k
        assert np.array_equal(np.asarray(a), G[k]), k


def test_linear_addressing_of_an_element_outside_its_dimension(tmp_path):
    src = """
PROGRAM T
IMPLICIT NONE
REAL(KIND=8), DIMENSION(2,3,4) :: a
REAL(KIND=8) :: r
a = 0.0
a(1,5,1) = 7.0
r = a(2,4,1)
END PROGRAM T
"""
    p = tmp_path / "t.f90"
    p.write_text(src)
    with pytest.raises(fs.FortranError):
        fs.Interp([p]).run_program(p, "T")
    v = fs.Interp([p], bounds="linear").run_program(p, "T").v
    a = v["A"].a
    # (1,5,1) is offset 0 + 2*4 = 8, i.e. element (1,2,2); (2,4,1) is (2,1,2)
    assert a[0, 1, 1] == 7.0 and np.count_nonzero(a) == 1 and v["R"] == 0.0
