"""The Fortran-subset translator that runs the reference's Fortran for the golden
vectors (tests/golden/f90py.py), checked on small programs of its own (CPU).

Each case is a few lines of Fortran whose compiled result is known: kinds and
mixed-kind arithmetic, integer division and MOD, integer powers, sequence
association of array arguments (including the out-of-bounds addressing the
reference's wtemp relies on), statement functions, internal procedures,
SELECT CASE, DO loops with exits, complex division as GCC forms it, the
poisoned start values that expose reads of storage never written, and the
line trace that lists the statements a run never executed.
"""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import f90py  # noqa: E402

FA = f90py.FArr


def _load(src, names, tmp_path):
    path = tmp_path / "t.f90"
    path.write_text(src)
    procs, _ = f90py.load([str(path)], names, math.atan, math.log)
    return procs


def i4(x):
    return np.array(x, dtype=np.int32)


def test_kinds_literals_and_integer_arithmetic(tmp_path):
    src = """
subroutine kinds(r8, r4w, idv, imd, neg, p3, b8)
  implicit none
  real(8), intent(out) :: r8, r4w, p3
  integer, intent(out) :: idv, imd, neg
  integer(1), intent(out) :: b8
  real(8), parameter :: tol = 1.e-2      ! a default-real literal
  integer(1) :: a
  r8 = 1.0d0/3.0d0
  r4w = tol
  idv = -7/2
  imd = mod(-7, 2)
  neg = int(-2.7d0)
  p3 = 1.1d0**3
  a = 100
  b8 = a + a                          ! integer(1) arithmetic wraps
end subroutine kinds
"""
    f = _load(src, ["kinds"], tmp_path)["kinds"]
    out = [np.array(0.0), np.array(0.0), i4(0), i4(0), i4(0), np.array(0.0), np.array(0, dtype=np.int8)]
    with np.errstate(over="ignore"):
        f(*out)
    r8, r4w, idv, imd, neg, p3, b8 = (x[()] for x in out)
    assert r8 == 1.0 / 3.0
    assert r4w == float(np.float32(1.e-2)) and r4w != 1.e-2
    assert (idv, imd, neg) == (-3, -1, -2)
    assert p3 == 1.1 * (1.1 * 1.1)                       # repeated squaring, not pow()
    assert b8 == np.int8(-56)


def test_sequence_association_and_out_of_bounds_addressing(tmp_path):
    src = """
subroutine fill(w, n, v)
  implicit none
  integer, intent(in) :: n
  real(8), intent(out) :: w(4, n)
  real(8), intent(in) :: v
  integer :: i, j
  do j = 1, n
     do i = 1, 4
        w(i, j) = v + 10*j + i
     enddo
  enddo
end subroutine fill

subroutine alias(out, n)
  implicit none
  integer, intent(in) :: n
  real(8), intent(out) :: out(4, n)
  real(8) :: wt(4, 2, n)
  integer :: isub
  wt = 0.0d0
  do isub = 1, 2
     call fill(wt(:, :, isub), n, 100.0d0*isub)
  enddo
  out(1:4, 1:n) = wt(1:4, 1:n, 1) + wt(1:4, 1:n, 2)
end subroutine alias
"""
    f = _load(src, ["alias"], tmp_path)["alias"]
    n = 4
    out = FA(np.zeros((4, n), order="F"), (1, 1))
    f(out, i4(n))
    w1 = np.array([[100 + 10 * j + i for j in range(1, n + 1)] for i in range(1, 5)], float)
    w2 = w1 + 100
    want = np.empty((4, n))
    for j in range(n):
        want[:, j] = (w1[:, j] if j < 2 else w2[:, j - 2]) + w2[:, j]
    assert np.array_equal(out.a, want)


def test_control_flow_statement_and_internal_functions(tmp_path):
    src = """
subroutine flow(n, res, cnt)
  implicit none
  integer, intent(in) :: n
  integer, intent(out) :: res, cnt
  integer :: i, k
  real(8) :: sq, x
  sq(x) = x*x
  res = 0
  cnt = 0
  do i = 1, n
     select case (mod(i, 4))
     case (0)
        cycle
     case (1:2)
        res = res + twice(i)
     case default
        res = res - 1
     end select
     if (res > 40) exit
     cnt = cnt + 1
  enddo
  k = 10
  do while (k > 1)
     k = k / 2
  enddo
  res = res * 100 + int(sq(dble(k)))
contains
  integer function twice(j)
    integer, intent(in) :: j
    twice = 2*j
  end function twice
end subroutine flow
"""
    f = _load(src, ["flow"], tmp_path)["flow"]
    res, cnt = i4(0), i4(0)
    f(i4(20), res, cnt)
    r, c = 0, 0
    for i in range(1, 21):
        m = i % 4
        if m == 0:
            continue
        r = r + 2 * i if m in (1, 2) else r - 1
        if r > 40:
            break
        c += 1
    k = 10
    while k > 1:
        k //= 2
    assert (res[()], cnt[()]) == (r * 100 + k * k, c)


def test_complex_division_as_compiled(tmp_path):
    src = """
subroutine cdiv(a, b, x, q1, q2, q3)
  implicit none
  complex*16, intent(in) :: a, b
  real(8), intent(in) :: x
  complex*16, intent(out) :: q1, q2, q3
  q1 = a / b
  q2 = a / x
  q3 = x / b
end subroutine cdiv
"""
    f = _load(src, ["cdiv"], tmp_path)["cdiv"]
    a, b, x = 1.3 - 0.7j, 0.2 + 2.5j, 3.14159265358979
    q = [np.array(0j), np.array(0j), np.array(0j)]
    f(np.array(a), np.array(b), np.array(x), *q)
    # Smith's method with the quotient formed by division; by a real divisor component-wise
    ratio = b.real / b.imag
    den = b.real * ratio + b.imag
    want1 = complex((a.real * ratio + a.imag) / den, (a.imag * ratio - a.real) / den)
    assert q[0][()] == want1
    assert q[1][()] == complex(a.real / x, a.imag / x)
    assert q[2][()] == complex((x * ratio + 0.0) / den, (0.0 * ratio - x) / den)


def test_unsupported_constructs_are_refused(tmp_path):
    src = """
subroutine bad(x)
  real(8), intent(out) :: x
  goto 10
10 x = 1.0d0
end subroutine bad
"""
    with pytest.raises(f90py.Unsupported):
        _load(src, ["bad"], tmp_path)


def test_poison_shows_reads_of_storage_never_written(tmp_path, monkeypatch):
    src = """
subroutine unset(x, n, b)
  implicit none
  real(8), intent(out) :: x
  integer, intent(out) :: n
  logical, intent(out) :: b
  real(8) :: w(3)
  integer :: k(2)
  w(1) = 1.0d0
  w(2) = 2.0d0
  x = w(1) + w(3)
  k(1) = 5
  n = k(2)
  b = btest(5, k(2))
end subroutine unset
"""
    f = _load(src, ["unset"], tmp_path)["unset"]
    x, n, b = np.array(0.0), i4(0), np.array(False)
    f(x, n, b)                                   # default: storage starts at zero
    assert (x[()], n[()], b[()]) == (1.0, 0, True)
    monkeypatch.setattr(f90py, "POISON", True)
    with pytest.raises(f90py.Undefined):         # a bit position never set
        f(x, n, b)
    assert np.isnan(x[()]) and n[()] == np.iinfo(np.int32).min


def test_line_trace_lists_the_statements_never_executed(tmp_path):
    src = """
subroutine pick(i, r)
  implicit none
  integer, intent(in) :: i
  integer, intent(out) :: r
  if (i > 0) then
     r = 1
  else
     r = -1
  endif
end subroutine pick
"""
    path = tmp_path / "t.f90"
    path.write_text(src)
    procs, tr = f90py.load([str(path)], ["pick"], math.atan, math.log)
    r = i4(0)
    with f90py.LineTrace() as t:
        procs["pick"](i4(3), r)
    ran, total, never = f90py.unexecuted(tr, t.hits)["pick"]
    assert r[()] == 1 and ran == total - 1 and len(never) == 1 and "-" in never[0]


def test_subscripts_beyond_the_storage_raise_undefined(tmp_path):
    """Out-of-bounds subscripts address the actual's storage as compiled code
    without bounds checks does; beyond that storage the result is undefined
    and the translator raises."""
    src = """
subroutine peek(w, n, i, x)
  implicit none
  integer, intent(in) :: n, i
  real(8), intent(in) :: w(2, n)
  real(8), intent(out) :: x
  x = w(1, i)
end subroutine peek
"""
    f = _load(src, ["peek"], tmp_path)["peek"]
    w = FA(np.asfortranarray(np.arange(8.0).reshape(2, 4, order="F")), (1, 1))
    x = np.array(0.0)
    f(w, i4(2), i4(4), x)                   # outside the dummy's (2, 2), inside the actual's storage
    assert x[()] == 6.0
    with pytest.raises(f90py.Undefined):
        f(w, i4(2), i4(5), x)
