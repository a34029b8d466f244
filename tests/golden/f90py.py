"""Run a subset of Fortran 90 from its source text under Python (test infrastructure).

The reference's tetrahedron-weight routines are Fortran for which neither
this container nor the GPU machine has a compiler.  To produce reference outputs
for them anyway, this module reads the Fortran source text at run time,
translates each requested procedure statement by statement into Python, and
executes the translation with numpy scalars and arrays standing in for the
Fortran variables:

* every variable keeps its declared kind — integer(1) → int8, integer →
  int32, default real → float32, real(8) / real*8 / double precision →
  float64, logical → bool — and the arithmetic of mixed kinds follows
  Fortran (the higher kind wins; integer division truncates; a default-real
  literal such as ``1.e-10`` is a float32 widened where it meets a double);
* scalars are 0-d numpy arrays and arrays are column-major views with their
  declared lower bounds, so arguments are passed by reference, and an array
  dummy of explicit shape is associated with its actual argument's storage
  from the actual's first element on (Fortran sequence association, which the
  reference relies on);
* control flow (DO, DO WHILE, IF, SELECT CASE, EXIT, CYCLE, RETURN, STOP),
  statement functions and internal procedures (CONTAINS) are translated one
  to one; WRITE and PRINT statements are dropped.

Only the constructs these routines use are supported; anything else raises
``Unsupported`` at translation time.  Intrinsic functions map to numpy, except
that ``atan`` and ``log`` (and their D-prefixed forms) call functions the
caller supplies, so a comparison can use the same implementations on both
sides.  Local variables and allocated arrays start at zero; with ``POISON``
set, their real and complex elements start at NaN and their integers at the
type's lowest value instead, and a bit test at a position outside the
integer raises ``Undefined``, so a result that depends on storage never
written (which compiled code leaves uninitialised) comes out NaN or raises.
Nothing of the reference's source is stored: the text is read from the
reference tree each time.
"""
from __future__ import annotations

import re

import numpy as np


class Unsupported(Exception):
    pass


class FortranStop(Exception):
    pass


class Undefined(IndexError):
    """The statements do something whose result compiled code leaves
    undefined: address outside an array's storage, or test a bit at a
    position outside the integer."""


# ----------------------------------------------------------------- runtime
I1, I4, I8, R4, R8, LG, C16 = np.int8, np.int32, np.int64, np.float32, np.float64, np.bool_, np.complex128


class Sect:
    """A subscript triplet lo:hi:step (None = the declared bound)."""
    __slots__ = ("lo", "hi", "st")

    def __init__(self, lo=None, hi=None, st=None):
        self.lo, self.hi, self.st = lo, hi, st


class FArr:
    """A Fortran array: numpy view (column-major) plus lower bounds."""
    __slots__ = ("a", "lb")

    def __init__(self, a, lb):
        self.a = a
        self.lb = tuple(int(x) for x in lb)

    def _np_index(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        if len(idx) != self.a.ndim:
            raise IndexError(f"rank {self.a.ndim} array indexed with {len(idx)} subscripts")
        out = []
        for d, (s, lb) in enumerate(zip(idx, self.lb)):
            n = self.a.shape[d]
            if isinstance(s, Sect):
                lo = lb if s.lo is None else int(s.lo)
                hi = lb + n - 1 if s.hi is None else int(s.hi)
                st = 1 if s.st is None else int(s.st)
                if st > 0:
                    if lo > hi:
                        out.append(slice(0, 0))
                        continue
                    if lo < lb or hi > lb + n - 1:
                        raise IndexError(f"section {lo}:{hi} outside {lb}:{lb + n - 1}")
                    out.append(slice(lo - lb, hi - lb + 1, st))
                else:
                    if lo < hi:
                        out.append(slice(0, 0))
                        continue
                    stop = hi - lb - 1
                    out.append(slice(lo - lb, None if stop < 0 else stop, st))
            else:
                i = int(s)
                if i < lb or i > lb + n - 1:
                    raise IndexError(f"subscript {i} outside {lb}:{lb + n - 1}")
                out.append(i - lb)
        return tuple(out)

    def _view(self, idx):
        try:
            return self.a[self._np_index(idx)]
        except IndexError:
            return self._unchecked(idx)

    def _unchecked(self, idx):
        """Subscripts beyond the declared bounds address memory the way compiled
        code without bounds checks does: from the declared strides, within the
        storage of the whole array (beyond it raises)."""
        if not isinstance(idx, tuple):
            idx = (idx,)
        starts, counts, steps, keep = [], [], [], []
        for d, (s, lb) in enumerate(zip(idx, self.lb)):
            n = self.a.shape[d]
            if isinstance(s, Sect):
                lo = lb if s.lo is None else int(s.lo)
                hi = lb + n - 1 if s.hi is None else int(s.hi)
                st = 1 if s.st is None else int(s.st)
                starts.append(lo - lb)
                counts.append(max(0, (hi - lo + st) // st))
                steps.append(st)
                keep.append(True)
            else:
                starts.append(int(s) - lb)
                counts.append(1)
                steps.append(1)
                keep.append(False)
        base, off0 = _base_and_offset(self.a)
        off = off0 + sum(k * self.a.strides[d] for d, k in enumerate(starts))
        strides = [self.a.strides[d] * steps[d] for d in range(self.a.ndim)]
        lo_b = off + sum(min(0, (c - 1) * s) for c, s in zip(counts, strides) if c > 0)
        hi_b = off + sum(max(0, (c - 1) * s) for c, s in zip(counts, strides) if c > 0)
        if lo_b < 0 or hi_b + self.a.itemsize > base.nbytes:
            raise Undefined("subscript outside the array's storage")
        v = np.ndarray(tuple(counts), dtype=self.a.dtype, buffer=base, offset=off, strides=tuple(strides))
        return v[tuple(slice(None) if k else 0 for k in keep)]

    def get(self, *idx):
        return self._view(idx)

    def set(self, idx, value):
        try:
            self.a[self._np_index(idx)] = value
        except IndexError:
            v = self._unchecked(idx)
            if v.ndim == 0:
                v[()] = value
            else:
                v[...] = value

    def sect(self, *idx):
        """The section as an FArr view (lower bounds 1), for actual arguments."""
        v = self._view(idx)
        return FArr(v, (1,) * v.ndim)

    def elem(self, *idx):
        """A 0-d view of one element (scalar actual argument / start of a sequence)."""
        ni = self._np_index(idx)
        return ElemRef(self, ni)


class ElemRef:
    """An array element passed as an actual argument: a 0-d view for a scalar
    dummy, or the start of sequence association for an array dummy."""
    __slots__ = ("arr", "ni")

    def __init__(self, arr, ni):
        self.arr, self.ni = arr, ni


def _base_and_offset(a):
    """numpy view → (base ndarray, byte offset of a's first element)."""
    base = a
    while isinstance(base.base, np.ndarray):
        base = base.base
    off = a.__array_interface__["data"][0] - base.__array_interface__["data"][0]
    return base, off


def assoc_array(actual, dtype, dims, lbs, intent=None):
    """Dummy array of explicit shape ``dims`` (None = assumed, from the
    actual) with lower bounds ``lbs``, associated with ``actual``."""
    if isinstance(actual, ElemRef):
        src = actual.arr.a
        first = src[tuple(slice(i, i + 1) for i in actual.ni)]
    elif isinstance(actual, FArr):
        src = actual.a
        first = src
    elif isinstance(actual, np.ndarray):
        src = actual
        first = src
    else:
        raise TypeError(f"array dummy given {type(actual)}")
    if src.dtype != np.dtype(dtype):
        raise TypeError(f"array dummy of {np.dtype(dtype)} given {src.dtype}")
    if dims is None or all(d is None for d in dims):
        if isinstance(actual, ElemRef):
            raise Unsupported("assumed-shape dummy given an element")
        return FArr(src, lbs)
    shape = tuple(int(d) for d in dims)
    size = int(np.prod(shape)) if shape else 1
    if isinstance(actual, (FArr, np.ndarray)) and src.flags.f_contiguous and src.size >= size:
        flat = src.reshape(-1, order="F")
        if np.shares_memory(flat, src) or src.size == 0:
            return FArr(flat[:size].reshape(shape, order="F"), lbs)
    if isinstance(actual, (FArr, np.ndarray)) and not src.flags.f_contiguous and intent == "in":
        # a non-contiguous section to an intent(in) dummy: compiled code passes
        # a contiguous copy (copy-in)
        if src.size < size:
            raise IndexError("dummy array larger than its actual argument")
        return FArr(np.asfortranarray(src).reshape(-1, order="F")[:size].reshape(shape, order="F"), lbs)
    # sequence association from the first element on, through the storage of
    # the whole array the actual belongs to (column-major)
    base, off = _base_and_offset(first)
    if not base.flags.f_contiguous and base.ndim > 1:
        raise Unsupported("sequence association into a non-contiguous array")
    item = base.itemsize
    if off + size * item > base.nbytes:
        raise IndexError("dummy array extends beyond its actual argument's storage")
    view = np.ndarray(shape, dtype=base.dtype, buffer=base, offset=off,
                      strides=tuple(item * int(np.prod(shape[:d])) for d in range(len(shape))))
    return FArr(view, lbs)


def assoc_scalar(actual, dtype):
    if isinstance(actual, ElemRef):
        a = actual.arr.a[tuple(slice(i, i + 1) for i in actual.ni)].reshape(())
        if a.dtype != np.dtype(dtype):
            return np.array(a, dtype=dtype)
        return a
    if isinstance(actual, np.ndarray) and actual.ndim == 0:
        if actual.dtype != np.dtype(dtype):
            return np.array(actual, dtype=dtype)
        return actual
    if isinstance(actual, FArr):
        raise TypeError("scalar dummy given an array")
    return np.array(actual, dtype=dtype)


# local variables and allocated arrays start at zero, or (POISON) at a value
# that shows a read before the first write
POISON = False


def _unset(dtype):
    dt = np.dtype(dtype)
    if POISON and np.issubdtype(dt, np.inexact):
        return np.nan
    if POISON and np.issubdtype(dt, np.integer):
        return np.iinfo(dt).min
    return 0


def unset_scalar(dtype):
    return np.array(_unset(dtype), dtype=dtype)


def new_array(dtype, bounds):
    lbs = [lo for lo, hi in bounds]
    shape = [max(0, int(hi) - int(lo) + 1) for lo, hi in bounds]
    a = np.zeros(shape, dtype=dtype, order="F")
    if _unset(dtype) != 0:
        a.fill(_unset(dtype))
    return FArr(a, lbs)


def val(x):
    """Value of an actual-argument object in an expression."""
    if isinstance(x, np.ndarray) and x.ndim == 0:
        return x[()]
    if isinstance(x, FArr):
        return x.a
    return x


def _is_int(x):
    return np.issubdtype(np.asarray(x).dtype, np.integer)


def _parts(x):
    x = np.asarray(x)
    if np.iscomplexobj(x):
        return x.real.astype(np.float64), x.imag.astype(np.float64), True
    return x.astype(np.float64), None, False


def _mkc(re_, im):
    re_ = np.asarray(re_, dtype=np.float64)
    r = np.empty(re_.shape, dtype=np.complex128)
    r.real = re_
    r.imag = im
    return r[()] if r.ndim == 0 else r


def mul(a, b):
    """Multiplication; with a complex operand as compiled code forms it
    without fused multiply-adds: (ar·br − ai·bi) + (ar·bi + ai·br)i, and
    component-wise when one operand is real."""
    if not (np.iscomplexobj(a) or np.iscomplexobj(b)):
        return a * b
    ar, ai, ca = _parts(a)
    br, bi, cb = _parts(b)
    if ca and cb:
        return _mkc(ar * br - ai * bi, ar * bi + ai * br)
    if ca:
        return _mkc(ar * br, ai * br)
    return _mkc(ar * br, ar * bi)


def _cdiv(a, b):
    """Complex division as GCC expands it for Fortran (Smith's method with the
    quotient formed by division), component-wise for a real divisor."""
    ar, ai, ca = _parts(a)
    br, bi, cb = _parts(b)
    if not cb:
        return _mkc(ar / br, ai / br)
    if ai is None:
        ai = np.zeros_like(ar)
    small = np.abs(br) < np.abs(bi)
    with np.errstate(all="ignore"):
        ratio_t = br / bi
        div_t = br * ratio_t + bi
        tr_t = (ar * ratio_t + ai) / div_t
        ti_t = (ai * ratio_t - ar) / div_t
        ratio_f = bi / br
        div_f = bi * ratio_f + br
        tr_f = (ai * ratio_f + ar) / div_f
        ti_f = (ai - ar * ratio_f) / div_f
    return _mkc(np.where(small, tr_t, tr_f), np.where(small, ti_t, ti_f))


def div(a, b):
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        return _cdiv(a, b)
    if _is_int(a) and _is_int(b):
        t = np.result_type(a, b)
        a = np.asarray(a).astype(np.int64)
        b = np.asarray(b).astype(np.int64)
        q = np.abs(a) // np.abs(b)
        q = np.where((a < 0) ^ (b < 0), -q, q)
        return q.astype(t)[()] if np.ndim(q) == 0 else q.astype(t)
    return a / b


def _powi(x, n):
    """x**n for an integer n as compiled code forms it: repeated squaring
    (x**2 = x·x, x**3 = x·(x·x), x**4 = (x·x)·(x·x)), not pow()."""
    if n < 0:
        return 1 / _powi(x, -n)
    if n == 0:
        return x * 0 + 1
    r = x if n % 2 else None
    n >>= 1
    while n:
        x = x * x
        if n % 2:
            r = x if r is None else r * x
        n >>= 1
    return r


def pw(a, b):
    if _is_int(b) and np.ndim(b) == 0:
        return _powi(a, int(b))
    return a ** b


def f_mod(a, p):
    if _is_int(a) and _is_int(p):
        return (a - div(a, p) * p)
    return np.fmod(a, p)


def f_int(x):
    return np.trunc(x).astype(I4)[()] if np.ndim(x) == 0 else np.trunc(x).astype(I4)


def f_nint(x):
    r = np.where(np.asarray(x) >= 0, np.floor(np.asarray(x) + 0.5), np.ceil(np.asarray(x) - 0.5)).astype(I4)
    return r[()] if np.ndim(r) == 0 else r


def f_sign(a, b):
    return np.abs(a) if b >= 0 else -np.abs(a)


def f_min(*xs):
    t = np.result_type(*xs)
    r = xs[0]
    for x in xs[1:]:
        r = np.minimum(r, x)
    return np.asarray(r, dtype=t)[()]


def f_max(*xs):
    t = np.result_type(*xs)
    r = xs[0]
    for x in xs[1:]:
        r = np.maximum(r, x)
    return np.asarray(r, dtype=t)[()]


def _bitpos(i, pos):
    if not 0 <= int(pos) < 8 * np.asarray(i).dtype.itemsize:
        raise Undefined(f"bit position {int(pos)}")
    return int(pos)


def f_btest(i, pos):
    return bool((int(i) >> _bitpos(i, pos)) & 1)


def f_ibset(i, pos):
    t = np.asarray(i).dtype
    return np.array(int(i) | (1 << _bitpos(i, pos))).astype(t)[()]


def f_ibclr(i, pos):
    t = np.asarray(i).dtype
    return np.array(int(i) & ~(1 << _bitpos(i, pos))).astype(t)[()]


def f_ibits(i, pos, ln):
    t = np.asarray(i).dtype
    return np.array((int(i) >> _bitpos(i, pos)) & ((1 << int(ln)) - 1)).astype(t)[()]


def f_matmul(a, b):
    """matmul of two rank-2 arrays, each element summed over k in ascending
    order from zero with separate multiplications and additions (the plain
    loop nest)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.ndim != 2 or b.ndim != 2 or a.shape[1] != b.shape[0]:
        raise Unsupported(f"matmul of shapes {a.shape} and {b.shape}")
    out = np.zeros((a.shape[0], b.shape[1]), dtype=np.result_type(a, b), order="F")
    for k in range(a.shape[1]):
        out = out + mul(a[:, k:k + 1], b[k:k + 1, :])
    return out


def f_size(a, dim=None):
    a = val(a)
    return I4(a.size if dim is None else a.shape[int(dim) - 1])


INTRINSICS = {
    "abs": "np.abs", "dabs": "np.abs", "iabs": "np.abs", "sqrt": "np.sqrt", "dsqrt": "np.sqrt",
    "mod": "f_mod", "int": "f_int", "nint": "f_nint", "sign": "f_sign", "dsign": "f_sign", "isign": "f_sign",
    "min": "f_min", "max": "f_max", "dmin1": "f_min", "dmax1": "f_max", "min0": "f_min", "max0": "f_max",
    "maxval": "np.max", "minval": "np.min", "sum": "np.sum", "size": "f_size", "matmul": "f_matmul",
    "btest": "f_btest", "ibset": "f_ibset", "ibclr": "f_ibclr", "ibits": "f_ibits",
    "dble": "R8", "dfloat": "R8", "float": "R4", "real": "_real", "atan": "_atan", "datan": "_atan",
    "log": "_log", "dlog": "_log", "allocated": "_allocated",
    "cmplx": "_cmplx", "dcmplx": "_cmplx", "conjg": "np.conj", "dconjg": "np.conj", "aimag": "np.imag",
    "dimag": "np.imag",
}


def _cmplx(re_, im=0.0, kind=None):
    if kind is None or int(kind) != 8:
        return np.complex64(complex(R4(re_), R4(im)))
    return C16(complex(float(re_), float(im)))


def _real(x, kind=None):
    return (R8 if kind is not None and int(kind) == 8 else R4)(x)


def _allocated(x):
    return x is not None


# ----------------------------------------------------------------- source
def _strip_comment(line):
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out).rstrip()


def logical_lines(text):
    """Comment-free, continuation-joined, lower-cased statements (strings kept)."""
    lines, cur = [], ""
    for raw in text.splitlines():
        s = _strip_comment(raw).strip()
        if not s:
            continue
        if cur:
            if s.startswith("&"):
                s = s[1:].lstrip()
            cur += " " + s
        else:
            cur = s
        if cur.endswith("&"):
            cur = cur[:-1].rstrip()
            continue
        lines.append(cur)
        cur = ""
    out = []
    for ln in lines:
        # lower-case outside string literals
        parts = re.split(r"('(?:[^']|'')*'|\"[^\"]*\")", ln)
        out.append("".join(p if i % 2 else p.lower() for i, p in enumerate(parts)))
    return out


_UNIT_START = re.compile(r"^(?:(?:real|integer|logical|double precision)(?:\s*\(\s*\d+\s*\)|\*\d+)?\s+)?"
                         r"(subroutine|function)\s+([a-z_]\w*)\s*(?:\((.*?)\))?\s*(?:result\s*\(\s*(\w+)\s*\))?$")


class Unit:
    def __init__(self, kind, name, args, result, rtype):
        self.kind, self.name, self.args, self.result, self.rtype = kind, name, args, result, rtype
        self.body = []          # statements
        self.internal = []      # Units (contains)


def parse_units(text):
    lines = logical_lines(text)
    units, stack = [], []
    i = 0
    in_interface = 0
    while i < len(lines):
        ln = lines[i]
        # interface blocks only declare external procedures: skipped
        if re.match(r"^(abstract\s+)?interface\b", ln):
            in_interface += 1
            i += 1
            continue
        if re.match(r"^end\s*interface\b", ln):
            in_interface -= 1
            i += 1
            continue
        if in_interface:
            i += 1
            continue
        m = _UNIT_START.match(ln)
        if m and not ln.startswith("end"):
            kind, name, args, result = m.group(1), m.group(2), m.group(3), m.group(4)
            rtype = None
            if kind == "function":
                pre = ln[:ln.index("function")].strip()
                rtype = pre or None
            u = Unit(kind, name, [a.strip() for a in args.split(",")] if args and args.strip() else [],
                     result, rtype)
            if stack:
                stack[-1].internal.append(u)
            else:
                units.append(u)
            stack.append(u)
        elif re.match(r"^end\s*(subroutine|function)\b", ln) or (ln == "end" and stack):
            stack.pop()
        elif ln == "contains":
            pass
        elif stack:
            stack[-1].body.append(ln)
        i += 1
    return {u.name: u for u in units}


# ------------------------------------------------------------- expressions
_TOKEN = re.compile(r"""
   (?P<ws>\s+)
 | (?P<dotop>\.(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
 | (?P<num>(?:\d+\.(?!(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv)\.)\d*|\.\d+|\d+)(?:[eEdD][+-]?\d+)?(?:_\w+)?)
 | (?P<name>[a-z_]\w*)
 | (?P<str>'(?:[^']|'')*'|"[^"]*")
 | (?P<op>\*\*|//|==|/=|<=|>=|\(/|/\)|[-+*/()<>,:=%\[\]])
""", re.X)


def tokenize(s):
    pos, out = 0, []
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise Unsupported(f"cannot tokenize {s[pos:]!r} in {s!r}")
        pos = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        out.append((k, m.group(k)))
    return out


class Node:
    def __init__(self, kind, *args):
        self.kind, self.args = kind, args


class ExprParser:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        return self.t[self.i + k] if self.i + k < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise Unsupported(f"expected {val!r}, got {tok!r}")
        self.i += 1
        return tok

    def parse(self):
        e = self.eqv()
        return e

    def eqv(self):
        e = self.orr()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.take()[1]
            e = Node("bin", "==" if op == ".eqv." else "!=", e, self.orr())
        return e

    def orr(self):
        e = self.andd()
        while self.peek()[1] == ".or.":
            self.take()
            e = Node("or", e, self.andd())
        return e

    def andd(self):
        e = self.nott()
        while self.peek()[1] == ".and.":
            self.take()
            e = Node("and", e, self.nott())
        return e

    def nott(self):
        if self.peek()[1] == ".not.":
            self.take()
            return Node("not", self.nott())
        return self.rel()

    REL = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
           "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}

    def rel(self):
        e = self.add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            e = Node("bin", op, e, self.add())
        return e

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            e = self.mul()
            e = Node("neg", e) if op == "-" else e
        else:
            e = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            e = Node("bin", op, e, self.mul())
        return e

    def mul(self):
        e = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            e = Node("bin", op, e, self.power())
        return e

    def power(self):
        b = self.unary_operand()
        if self.peek()[1] == "**":
            self.take()
            return Node("pow", b, self.power_rhs())
        return b

    def power_rhs(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            e = self.power()
            return Node("neg", e) if op == "-" else e
        return self.power()

    def unary_operand(self):
        if self.peek()[1] in ("+", "-"):     # a*-b (a gfortran extension)
            op = self.take()[1]
            e = self.power()
            return Node("neg", e) if op == "-" else e
        return self.primary()

    def primary(self):
        k, v = self.take()
        if k == "num":
            return Node("num", v)
        if k == "dotop" and v in (".true.", ".false."):
            return Node("lgl", v == ".true.")
        if k == "str":
            return Node("str", v)
        if v == "(":
            e = self.parse()
            self.take(")")
            return Node("paren", e)
        if v in ("(/", "["):
            items = [self.parse()]
            while self.peek()[1] == ",":
                self.take()
                items.append(self.parse())
            self.take("/)" if v == "(/" else "]")
            return Node("ctor", items)
        if k == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    args.append(self.subscript())
                    while self.peek()[1] == ",":
                        self.take()
                        args.append(self.subscript())
                self.take(")")
                return Node("call", v, args)
            return Node("name", v)
        raise Unsupported(f"unexpected token {v!r}")

    def subscript(self):
        # expr | [expr] : [expr] [: expr] | name = expr (keyword argument)
        if self.peek()[0] == "name" and self.peek(1)[1] == "=" and self.peek(2)[1] != "=":
            kw = self.take()[1]
            self.take("=")
            return Node("kw", kw, self.parse())
        lo = hi = st = None
        if self.peek()[1] != ":":
            lo = self.parse()
            if self.peek()[1] != ":":
                return lo
        self.take(":")
        if self.peek()[1] not in (":", ",", ")"):
            hi = self.parse()
        if self.peek()[1] == ":":
            self.take()
            st = self.parse()
        return Node("sect", lo, hi, st)


def parse_expr(s):
    p = ExprParser(tokenize(s))
    e = p.parse()
    if p.i != len(p.t):
        raise Unsupported(f"trailing tokens in {s!r}: {p.t[p.i:]}")
    return e


# ------------------------------------------------------------ declarations
_TYPES = [
    (r"integer\s*\(\s*(?:kind\s*=\s*)?1\s*\)|integer\*1", "I1"),
    (r"integer\s*\(\s*(?:kind\s*=\s*)?8\s*\)|integer\*8", "I8"),
    (r"integer\s*\(\s*(?:kind\s*=\s*)?4\s*\)|integer\*4|integer", "I4"),
    (r"real\s*\(\s*(?:kind\s*=\s*)?8\s*\)|real\*8|double\s+precision", "R8"),
    (r"real\s*\(\s*(?:kind\s*=\s*)?4\s*\)|real\*4|real", "R4"),
    (r"logical\s*\(\s*\d+\s*\)|logical", "LG"),
    (r"complex\s*\(\s*(?:kind\s*=\s*)?8\s*\)|complex\*16|double\s+complex", "C16"),
]


def match_type(s):
    for pat, t in _TYPES:
        m = re.match(r"^(?:" + pat + r")(?![a-z0-9_])", s)
        if m:
            return t, s[m.end():]
    return None, s


def split_top(s, sep=","):
    out, depth, cur, q = [], 0, "", None
    for ch in s:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return [x.strip() for x in out]


class Var:
    def __init__(self, name, typ):
        self.name, self.typ = name, typ
        self.dims = None        # list of (lo_expr, hi_expr) strings; hi None = assumed / deferred
        self.param = None       # initial value expression (parameter)
        self.init = None
        self.intent = None
        self.alloc = False
        self.is_arg = False
        self.external = False


# --------------------------------------------------------------- translator
class Translator:
    def __init__(self, units, atan, log):
        self.units = units
        self.ns = {"np": np, "I1": I1, "I4": I4, "I8": I8, "R4": R4, "R8": R8, "LG": LG, "C16": C16, "Sect": Sect,
                   "FArr": FArr, "ElemRef": ElemRef, "assoc_array": assoc_array, "assoc_scalar": assoc_scalar,
                   "new_array": new_array, "unset_scalar": unset_scalar, "val": val, "div": div, "mul": mul,
                   "pw": pw, "f_mod": f_mod, "f_int": f_int,
                   "f_nint": f_nint, "f_sign": f_sign, "f_min": f_min, "f_max": f_max, "f_btest": f_btest,
                   "f_ibset": f_ibset, "f_ibclr": f_ibclr, "f_ibits": f_ibits, "f_size": f_size,
                   "f_matmul": f_matmul,
                   "_real": _real, "_allocated": _allocated, "FortranStop": FortranStop,
                   "_cmplx": _cmplx,
                   "_atan": lambda x: (np.arctan(x) if np.iscomplexobj(x) else R8(atan(float(x)))),
                   "_log": lambda x: (np.log(x) if np.iscomplexobj(x) else R8(log(float(x))))}
        self.done = set()
        self.sources = {}       # unit name -> generated Python source

    def procedure(self, name):
        if name not in self.done:
            self.translate(self.units[name])
        return self.ns["f_" + name]

    # -- per-unit
    def translate(self, u, host_vars=None, indent=0):
        src = self.emit_unit(u, host_vars or {}, indent)
        if indent == 0:
            code = "\n".join(src)
            self.sources[u.name] = code
            try:
                exec(compile(code, f"<f90:{u.name}>", "exec"), self.ns)
            except SyntaxError as e:
                raise Unsupported(f"generated code for {u.name} does not compile: {e}\n{code}")
            self.done.add(u.name)
        return src

    def emit_unit(self, u, host_vars, indent):
        vars_ = dict(host_vars)
        local = {}
        stmt_funcs = []
        body_start = 0
        args = u.args
        # declarations
        for n, ln in enumerate(u.body):
            if ln.startswith("implicit"):
                continue
            if re.match(r"^(external|intrinsic)\b", ln):
                for nm in split_top(ln.split(None, 1)[1].replace("::", "")):
                    if nm in local:
                        local[nm].external = True
                continue
            if re.match(r"^(use|save)\b", ln):
                continue
            t, rest = match_type(ln)
            if t is not None and (rest.lstrip().startswith("::") or rest.startswith(",")
                                  or re.match(r"^\s+[a-z_]", rest)):
                self.declare(rest, t, local)
                continue
            # statement function: name(args) = expr, name declared as a scalar
            m = re.match(r"^([a-z_]\w*)\s*\(([^()]*)\)\s*=(?!=)(.*)$", ln)
            if m and m.group(1) in local and local[m.group(1)].dims is None and not local[m.group(1)].is_arg:
                stmt_funcs.append((m.group(1), [a.strip() for a in m.group(2).split(",")], m.group(3).strip()))
                continue
            body_start = n
            break
        else:
            body_start = len(u.body)
        exec_lines = list(u.body[body_start:])
        for a in args:
            if a in local:
                local[a].is_arg = True
            else:
                local[a] = Var(a, "R4" if a[0] in "abcdefghopqrstuvwxyz" else "I4")   # implicit typing
                local[a].is_arg = True
        if u.kind == "function":
            rname = u.result or u.name
            if rname not in local:
                t, _ = match_type(u.rtype or "")
                local[rname] = Var(rname, t or "R8")
        for k, v in local.items():
            vars_[k] = v
        sf_names = {s[0] for s in stmt_funcs}
        self.cur_vars = vars_
        self.cur_sf = sf_names
        self.cur_internal = {iu.name for iu in u.internal}
        pad = "    " * indent
        out = [f"{pad}def f_{u.name}({', '.join('a_' + a for a in args)}):"]
        p1 = pad + "    "
        # dummies first (bounds may refer to other dummies), then locals in order
        order = ([a for a in args if local[a].dims is None] + [a for a in args if local[a].dims is not None]
                 + [k for k in local if k not in args])
        for k in order:
            v = local[k]
            if v.external or k in sf_names:
                continue
            if v.param is not None:
                continue
            out.extend(self.emit_decl(v, p1))
        # parameters before everything else would need their values in bounds:
        params = [v for v in local.values() if v.param is not None]
        pre = []
        for v in params:
            pre.append(f"{p1}v_{v.name} = np.array({self.expr(parse_expr(v.param))}, dtype={v.typ})"
                       if v.dims is None else
                       f"{p1}v_{v.name} = FArr(np.array({self.expr(parse_expr(v.param))}, dtype={v.typ}, order='F'), "
                       f"({', '.join(self.expr(parse_expr(lo)) for lo, hi in v.dims)},))")
        out[1:1] = pre
        for name, sargs, sexpr in stmt_funcs:
            saved = dict(self.cur_vars)
            for a in sargs:
                self.cur_vars[a] = Var(a, vars_[a].typ if a in vars_ else "I4")
                self.cur_vars[a].sfarg = True
            out.append(f"{p1}def f_{name}({', '.join('s_' + a for a in sargs)}):")
            for a in sargs:
                out.append(f"{p1}    v_{a} = np.array(s_{a}, dtype={self.cur_vars[a].typ})")
            out.append(f"{p1}    return {local[name].typ}({self.expr(parse_expr(sexpr))})")
            self.cur_vars = saved
        for iu in u.internal:
            out.extend(self.emit_unit(iu, vars_, indent + 1))
            self.cur_vars = vars_
            self.cur_sf = sf_names
            self.cur_internal = {x.name for x in u.internal}
        body = self.block(exec_lines, indent + 1, u)
        out.extend(body)
        if u.kind == "function":
            out.append(f"{p1}return v_{u.result or u.name}[()]")
        else:
            out.append(f"{p1}return None")
        return out

    def declare(self, rest, typ, local):
        if "::" in rest:
            attrs, ents = rest.split("::", 1)
        else:
            attrs, ents = "", rest
        attrs = [a.strip() for a in split_top(attrs.lstrip(",")) if a.strip()]
        dims_attr = None
        intent = None
        param = alloc = False
        for a in attrs:
            if a.startswith("intent"):
                intent = a[a.index("(") + 1:a.rindex(")")].strip()
            elif a == "parameter":
                param = True
            elif a == "allocatable":
                alloc = True
            elif a.startswith("dimension"):
                dims_attr = a[a.index("(") + 1:a.rindex(")")]
            elif a in ("save", "target", "optional", "pointer", "external", "intrinsic"):
                continue
            else:
                raise Unsupported(f"attribute {a}")
        for ent in split_top(ents):
            if not ent:
                continue
            init = None
            if "=" in ent and not ent.split("=", 1)[0].strip().endswith(("<", ">", "/")):
                ent, init = [x.strip() for x in ent.split("=", 1)]
            m = re.match(r"^([a-z_]\w*)\s*(?:\((.*)\))?$", ent)
            if not m:
                raise Unsupported(f"declaration entity {ent!r}")
            v = Var(m.group(1), typ)
            d = m.group(2) if m.group(2) is not None else dims_attr
            if d is not None:
                v.dims = []
                for dd in split_top(d):
                    if dd in (":", "*"):
                        v.dims.append(("1", None))
                    elif ":" in dd:
                        lo, hi = [x.strip() for x in dd.split(":", 1)]
                        v.dims.append((lo or "1", hi or None))
                    else:
                        v.dims.append(("1", dd))
            v.intent, v.alloc = intent, alloc
            if param:
                v.param = init
            else:
                v.init = init
            local[v.name] = v

    def emit_decl(self, v, p):
        t = v.typ
        if v.is_arg:
            if v.dims is None:
                return [f"{p}v_{v.name} = assoc_scalar(a_{v.name}, {t})"]
            los = ", ".join(self.expr(parse_expr(lo)) for lo, hi in v.dims)
            if any(hi is None for lo, hi in v.dims):
                return [f"{p}v_{v.name} = assoc_array(a_{v.name}, {t}, None, ({los},))"]
            his = ", ".join(f"({self.expr(parse_expr(hi))}) - ({self.expr(parse_expr(lo))}) + 1"
                            for lo, hi in v.dims)
            return [f"{p}v_{v.name} = assoc_array(a_{v.name}, {t}, ({his},), ({los},), {v.intent!r})"]
        if v.alloc:
            return [f"{p}v_{v.name} = None"]
        if v.dims is None:
            if not v.init:
                return [f"{p}v_{v.name} = unset_scalar({t})"]
            return [f"{p}v_{v.name} = np.array({self.expr(parse_expr(v.init))}, dtype={t})"]
        bounds = ", ".join(f"({self.expr(parse_expr(lo))}, {self.expr(parse_expr(hi))})" for lo, hi in v.dims)
        out = [f"{p}v_{v.name} = new_array({t}, [{bounds}])"]
        if v.init:
            out.append(f"{p}v_{v.name}.a[...] = {self.expr(parse_expr(v.init))}")
        return out

    # -- expressions
    def is_array(self, name):
        v = self.cur_vars.get(name)
        return v is not None and (v.dims is not None) and not getattr(v, "sfarg", False)

    def is_var(self, name):
        v = self.cur_vars.get(name)
        return v is not None and not v.external and name not in self.cur_sf

    def literal(self, s):
        s2 = s.split("_")[0]
        kind = s.split("_")[1] if "_" in s else None
        if re.fullmatch(r"\d+", s2):
            return f"{'I8' if kind == '8' else 'I4'}({s2})"
        if "d" in s2:
            return f"R8({float(s2.replace('d', 'e'))!r})"
        if kind == "8":
            return f"R8({float(s2)!r})"
        return f"R4({float(s2)!r})"

    def expr(self, n, ctx="val"):
        k = n.kind
        a = n.args
        if k == "num":
            return self.literal(a[0])
        if k == "lgl":
            return "LG(True)" if a[0] else "LG(False)"
        if k == "str":
            return repr(a[0][1:-1])
        if k == "paren":
            return f"({self.expr(a[0])})"
        if k == "neg":
            return f"(-{self.expr(a[0])})"
        if k == "not":
            return f"(not {self.expr(a[0])})"
        if k == "and":
            return f"({self.expr(a[0])} and {self.expr(a[1])})"
        if k == "or":
            return f"({self.expr(a[0])} or {self.expr(a[1])})"
        if k == "pow":
            return f"pw({self.expr(a[0])}, {self.expr(a[1])})"
        if k == "bin":
            op, l, r = a
            if op == "/":
                return f"div({self.expr(l)}, {self.expr(r)})"
            if op == "*":
                return f"mul({self.expr(l)}, {self.expr(r)})"
            return f"({self.expr(l)} {op} {self.expr(r)})"
        if k == "ctor":
            return f"np.array([{', '.join(self.expr(x) for x in a[0])}])"
        if k == "name":
            nm = a[0]
            if self.is_array(nm):
                return f"v_{nm}.a" if ctx == "val" else f"v_{nm}"
            if self.is_var(nm):
                return f"v_{nm}[()]" if ctx == "val" else f"v_{nm}"
            raise Unsupported(f"unknown name {nm}")
        if k == "call":
            nm, args = a
            if self.is_array(nm):
                subs = ", ".join(self.subscr(x) for x in args)
                whole = any(x.kind == "sect" for x in args)
                if ctx == "arg":
                    return f"v_{nm}.sect({subs})" if whole else f"v_{nm}.elem({subs})"
                return f"v_{nm}.get({subs})"
            if nm in self.cur_sf:
                return f"f_{nm}({', '.join(self.expr(x) for x in args)})"
            if nm in INTRINSICS and nm not in self.cur_internal and not (nm in self.cur_vars and
                                                                      self.cur_vars[nm].external):
                fn = INTRINSICS[nm]
                vals = []
                for x in args:
                    if x.kind == "kw":
                        vals.append(self.expr(x.args[1]))
                    elif nm in ("allocated", "size"):
                        vals.append(self.expr(x, ctx="arg"))
                    else:
                        vals.append(self.expr(x))
                return f"{fn}({', '.join(vals)})"
            # user function (internal or external)
            return f"{self.fn_ref(nm)}({', '.join(self.actual(x) for x in args)})"
        if k == "sect":
            raise Unsupported("section outside a subscript")
        raise Unsupported(f"node {k}")

    def subscr(self, x):
        if x.kind == "sect":
            lo, hi, st = x.args
            return (f"Sect({self.expr(lo) if lo else None}, {self.expr(hi) if hi else None}, "
                    f"{self.expr(st) if st else None})")
        return self.expr(x)

    def actual(self, x):
        if x.kind == "name" and (self.is_array(x.args[0]) or self.is_var(x.args[0])):
            return self.expr(x, ctx="arg")
        if x.kind == "call" and self.is_array(x.args[0]):
            return self.expr(x, ctx="arg")
        return f"np.array({self.expr(x)})"

    def fn_ref(self, nm):
        if nm in self.cur_internal:
            return f"f_{nm}"
        return f"_proc({nm!r})"

    # -- statements
    def block(self, lines, ind, u):
        out = []
        p = "    " * ind
        i = 0
        while i < len(lines):
            ln = lines[i]
            if re.match(r"^if\s*\(", ln) and ln.rstrip().endswith("then") and self._if_then(ln):
                # collect the IF construct
                depth, j, parts, cond = 1, i + 1, [], self._cond(ln)
                cur_cond, cur = cond, []
                while j < len(lines):
                    l2 = lines[j]
                    if re.match(r"^if\s*\(", l2) and l2.rstrip().endswith("then") and self._if_then(l2):
                        depth += 1
                    elif re.match(r"^end\s*if\b", l2):
                        depth -= 1
                        if depth == 0:
                            break
                    elif depth == 1 and re.match(r"^else\s*if\s*\(", l2):
                        parts.append((cur_cond, cur))
                        cur_cond, cur = self._cond(l2[l2.index("if"):]), []
                        j += 1
                        continue
                    elif depth == 1 and re.match(r"^else$", l2):
                        parts.append((cur_cond, cur))
                        cur_cond, cur = None, []
                        j += 1
                        continue
                    cur.append(l2)
                    j += 1
                parts.append((cur_cond, cur))
                for n, (c, blk) in enumerate(parts):
                    kw = "if" if n == 0 else ("elif" if c is not None else "else")
                    out.append(f"{p}{kw} {self.expr(parse_expr(c))}:" if c is not None else f"{p}else:")
                    sub = self.block(blk, ind + 1, u)
                    out.extend(sub or [f"{p}    pass"])
                i = j + 1
                continue
            m = re.match(r"^do\s+while\s*\((.*)\)$", ln)
            if m or re.match(r"^do\s+[a-z_]\w*\s*=", ln) or ln == "do":
                depth, j = 1, i + 1
                while j < len(lines):
                    if re.match(r"^do\b", lines[j]):
                        depth += 1
                    elif re.match(r"^end\s*do\b", lines[j]):
                        depth -= 1
                        if depth == 0:
                            break
                    j += 1
                inner = lines[i + 1:j]
                if m:
                    out.append(f"{p}while {self.expr(parse_expr(m.group(1)))}:")
                elif ln == "do":
                    out.append(f"{p}while True:")
                else:
                    mm = re.match(r"^do\s+([a-z_]\w*)\s*=\s*(.*)$", ln)
                    var = mm.group(1)
                    parts = split_top(mm.group(2))
                    lo, hi = self.expr(parse_expr(parts[0])), self.expr(parse_expr(parts[1]))
                    st = self.expr(parse_expr(parts[2])) if len(parts) > 2 else "I4(1)"
                    out.append(f"{p}for _v in _frange({lo}, {hi}, {st}):")
                    out.append(f"{p}    v_{var}[()] = _v")
                sub = self.block(inner, ind + 1, u)
                out.extend(sub or [f"{p}    pass"])
                i = j + 1
                continue
            m = re.match(r"^select\s+case\s*\((.*)\)$", ln)
            if m:
                depth, j = 1, i + 1
                cases, cur_sel, cur = [], None, []
                while j < len(lines):
                    l2 = lines[j]
                    if re.match(r"^select\s+case", l2):
                        depth += 1
                    elif re.match(r"^end\s*select", l2):
                        depth -= 1
                        if depth == 0:
                            break
                    elif depth == 1 and re.match(r"^case\b", l2):
                        if cur_sel is not None:
                            cases.append((cur_sel, cur))
                        cur_sel, cur = l2, []
                        j += 1
                        continue
                    cur.append(l2)
                    j += 1
                if cur_sel is not None:
                    cases.append((cur_sel, cur))
                sv = f"_sel{ind}"
                out.append(f"{p}{sv} = {self.expr(parse_expr(m.group(1)))}")
                first = True
                default = None
                for sel, blk in cases:
                    if re.match(r"^case\s+default", sel):
                        default = blk
                        continue
                    items = split_top(sel[sel.index("(") + 1:sel.rindex(")")])
                    conds = []
                    for it in items:
                        if ":" in it:
                            lo, hi = [x.strip() for x in it.split(":", 1)]
                            c = []
                            if lo:
                                c.append(f"{sv} >= {self.expr(parse_expr(lo))}")
                            if hi:
                                c.append(f"{sv} <= {self.expr(parse_expr(hi))}")
                            conds.append("(" + " and ".join(c) + ")")
                        else:
                            conds.append(f"{sv} == {self.expr(parse_expr(it))}")
                    out.append(f"{p}{'if' if first else 'elif'} {' or '.join(conds)}:")
                    first = False
                    out.extend(self.block(blk, ind + 1, u) or [f"{p}    pass"])
                if default is not None:
                    if first:
                        out.append(f"{p}if True:")
                    else:
                        out.append(f"{p}else:")
                    out.extend(self.block(default, ind + 1, u) or [f"{p}    pass"])
                i = j + 1
                continue
            out.extend(self.simple(ln, p, u))
            i += 1
        return out

    def _if_then(self, ln):
        c = self._cond(ln)
        rest = ln[ln.index("(") + len(c) + 2:].strip()
        return rest == "then"

    def _cond(self, ln):
        s = ln[ln.index("(") + 1:]
        depth = 1
        for n, ch in enumerate(s):
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    return s[:n]
        raise Unsupported(f"unbalanced {ln!r}")

    def simple(self, ln, p, u):
        if ln in ("continue",):
            return [f"{p}pass"]
        if ln == "return":
            if u.kind == "function":
                return [f"{p}return v_{u.result or u.name}[()]"]
            return [f"{p}return None"]
        if ln == "exit":
            return [f"{p}break"]
        if ln == "cycle":
            return [f"{p}continue"]
        if ln.startswith("stop"):
            return [f"{p}raise FortranStop({ln[4:].strip()!r})"]
        if re.match(r"^(write|print|flush)\b", ln):
            return [f"{p}pass"]
        m = re.match(r"^if\s*\(", ln)
        if m:
            c = self._cond(ln)
            rest = ln[ln.index("(") + len(c) + 2:].strip()
            inner = self.simple(rest, p + "    ", u)
            return [f"{p}if {self.expr(parse_expr(c))}:"] + inner
        m = re.match(r"^call\s+([a-z_]\w*)\s*(?:\((.*)\))?$", ln)
        if m:
            nm = m.group(1)
            args = split_top(m.group(2)) if m.group(2) and m.group(2).strip() else []
            acts = ", ".join(self.actual(parse_expr(x)) for x in args)
            return [f"{p}{self.fn_ref(nm)}({acts})"]
        m = re.match(r"^allocate\s*\((.*)\)$", ln)
        if m:
            out = []
            for ent in split_top(m.group(1)):
                mm = re.match(r"^([a-z_]\w*)\s*\((.*)\)$", ent)
                v = self.cur_vars[mm.group(1)]
                bounds = []
                for dd in split_top(mm.group(2)):
                    if ":" in dd:
                        lo, hi = dd.split(":", 1)
                    else:
                        lo, hi = "1", dd
                    bounds.append(f"({self.expr(parse_expr(lo))}, {self.expr(parse_expr(hi))})")
                out.append(f"{p}v_{v.name} = new_array({v.typ}, [{', '.join(bounds)}])")
            return out
        m = re.match(r"^deallocate\s*\((.*)\)$", ln)
        if m:
            return [f"{p}v_{x} = None" for x in split_top(m.group(1))]
        # assignment
        lhs, rhs = self._split_assign(ln)
        if lhs is None:
            raise Unsupported(f"statement {ln!r}")
        rv = self.expr(parse_expr(rhs))
        ln_node = parse_expr(lhs)
        if ln_node.kind == "name":
            nm = ln_node.args[0]
            if self.is_array(nm):
                return [f"{p}v_{nm}.a[...] = {rv}"]
            return [f"{p}v_{nm}[()] = {rv}"]
        if ln_node.kind == "call" and self.is_array(ln_node.args[0]):
            subs = ", ".join(self.subscr(x) for x in ln_node.args[1])
            return [f"{p}v_{ln_node.args[0]}.set(({subs},), {rv})"]
        raise Unsupported(f"assignment target {lhs!r}")

    def _split_assign(self, ln):
        depth = 0
        for n, ch in enumerate(ln):
            if ch in "([":
                depth += 1
            elif ch in ")]":
                depth -= 1
            elif ch == "=" and depth == 0 and ln[n + 1:n + 2] != "=" and ln[n - 1:n] not in "<>/=":
                return ln[:n].strip(), ln[n + 1:].strip()
        return None, None


def _frange(lo, hi, st):
    lo, hi, st = int(lo), int(hi), int(st)
    n = max(0, (hi - lo + st) // st) if st > 0 else max(0, (lo - hi - st) // (-st))
    return [lo + k * st for k in range(n)]


class LineTrace:
    """Context manager recording which lines of the translated procedures
    run (``hits``: {unit name: set of line numbers of its generated source})."""

    def __init__(self):
        import collections
        self.hits = collections.defaultdict(set)

    def _global(self, frame, event, arg):
        if not frame.f_code.co_filename.startswith("<f90:"):
            return None
        return self._local

    def _local(self, frame, event, arg):
        if event == "line":
            self.hits[frame.f_code.co_filename[5:-1]].add(frame.f_lineno)
        return self._local

    def __enter__(self):
        import sys
        sys.settrace(self._global)
        return self

    def __exit__(self, *exc):
        import sys
        sys.settrace(None)
        return False


def unexecuted(tr, hits):
    """{unit name: (executed, executable, [generated lines never run])} for
    every procedure ``tr`` translated, given ``LineTrace.hits``."""
    out = {}
    for name, src in sorted(tr.sources.items()):
        lines, stack = set(), [compile(src, f"<f90:{name}>", "exec")]
        while stack:
            c = stack.pop()
            lines.update(ln for _, _, ln in c.co_lines() if ln)
            stack.extend(x for x in c.co_consts if hasattr(x, "co_lines"))
        text = src.split("\n")
        lines = {ln for ln in lines if not text[ln - 1].lstrip().startswith("def ")}
        miss = sorted(lines - hits.get(name, set()))
        out[name] = (len(lines) - len(miss), len(lines), [text[ln - 1].strip() for ln in miss])
    return out


LOADED = []            # every Translator load() made, for coverage reports


def load(paths, names, atan, log):
    """Translate the procedures ``names`` (and whatever they call, on demand)
    from the Fortran files ``paths``; returns {name: callable}."""
    units = {}
    for path in paths:
        with open(path) as f:
            units.update(parse_units(f.read()))
    tr = Translator(units, atan, log)
    LOADED.append(tr)
    tr.ns["_frange"] = _frange
    tr.ns["_proc"] = lambda nm: tr.procedure(nm)
    return {n: tr.procedure(n) for n in names}, tr
