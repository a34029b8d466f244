"""ctypes front end of the oracle's weight restatement (test infrastructure).

Parity pinned against the reference's own statements: with no Fortran compiler
here, tests/golden/make_weights_golden.py executes the reference's
bz_calcqdepw_par2 and its callees from their Fortran text (tests/golden/f90py.py)
on seeded inputs, and this restatement reproduces those kcw bit for bit
(tests/test_oracle_weights_golden.py) except at the reference's own layout bug
for 7- and 8-node polyhedra (frequencies from the third on); known answers
(tests/test_oracle_*.py) check the integrals themselves.

``bz_calcqdepw_par2`` mirrors the f2py call of the reference
(``kcw = ft.bz_calcqdepw_par2(enk, ef, kqid, ncg, nomx, numin, omega, tetc)``,
pygw.py:3443, for_tetrahedra.f90:390): array sizes are inferred from the
shapes, arrays are Fortran-ordered, ``kqid``/``tetc`` are 0-based.
``bz_calcqdepw_par3`` mirrors ``ft.bz_calcqdepw_par3(enk, ef, kqid, ncg, nomx,
numin, dUl, omega, tetc)`` (pygw.py:3441, for_tetrahedra.f90:466).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import build

_LIBS = {}
STAT_NAMES = (["calls"] + [f"nnod{i}" for i in range(9)] + [f"equiv{i}" for i in (4, 6, 8, 10, 16)]
              + ["taylor", "exact", "zero_vol", "big_weight_warn", "big_weight_zeroed"])


def _lib(libm=False):
    key = "libm" if libm else "portable"
    if key not in _LIBS:
        paths = build()
        lib = ctypes.CDLL(paths["liboracle_weights_libm.so" if libm else "liboracle_weights.so"])
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_longlong)
        lib.oracle_bz_calcqdepw_par2.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ip, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ip, ctypes.c_int, dp,
                                                 ctypes.c_int, lp]
        lib.oracle_bz_calcqdepw_par2.restype = ctypes.c_int
        lib.oracle_bz_calcqdepw_par3.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ip, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, dp, ctypes.c_int, ip,
                                                 ctypes.c_int, dp, ctypes.c_int]
        lib.oracle_bz_calcqdepw_par3.restype = ctypes.c_int
        lib.oracle_convw1t.argtypes = [dp, dp, ctypes.c_double, dp, ctypes.c_int, dp, lp]
        lib.oracle_convw1t.restype = ctypes.c_int
        lib.oracle_generictetra.argtypes = [dp, dp, dp, dp, ctypes.c_int, dp]
        lib.oracle_generictetra.restype = ctypes.c_int
        lib.oracle_portable_math.argtypes = [dp, ctypes.c_int, dp, dp]
        lib.oracle_portable_math.restype = None
        lib.oracle_set_reference_layout.argtypes = [ctypes.c_int]
        lib.oracle_set_reference_layout.restype = None
        _LIBS[key] = lib
    return _LIBS[key]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def bz_calcqdepw_par2(enk, ef, kqid, ncg, nomx, numin, omega, tetc, nthreads=0, libm=False, return_stats=False):
    """Restated weights; returns ``kcw[ncg+nomx+1, nbnd-ncg-numin, nkp, nom]`` (F order)."""
    enk = np.asfortranarray(enk, dtype=np.float64)
    kqid = np.ascontiguousarray(kqid, dtype=np.int32)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    tetc = np.asfortranarray(tetc, dtype=np.int32)
    nbnd, nkp = enk.shape
    nom = omega.shape[0]
    ntet = tetc.shape[1]
    nb1, nb2 = ncg + nomx + 1, nbnd - ncg - numin
    kcw = np.zeros((nb1, nb2, nkp, nom), order="F")
    stats = np.zeros(20, dtype=np.int64)
    st = _lib(libm).oracle_bz_calcqdepw_par2(_dp(enk), nbnd, nkp, float(ef), _ip(kqid), ncg, nomx, numin, _dp(omega),
                                             nom, _ip(tetc), ntet, _dp(kcw), int(nthreads),
                                             stats.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
    if st < 0:
        raise ValueError("oracle_bz_calcqdepw_par2: bad sizes")
    if return_stats:
        return kcw, int(st), dict(zip(STAT_NAMES, stats.tolist()))
    return kcw


def bz_calcqdepw_par3(enk, ef, kqid, ncg, nomx, numin, dUl, omega, tetc, nthreads=0, libm=False):
    """Restated SVD-basis weights (for_tetrahedra.f90:466-542); ``dUl[nom, nl]``;
    returns ``kcw[ncg+nomx+1, nbnd-ncg-numin, nkp, nl]`` (F order)."""
    enk = np.asfortranarray(enk, dtype=np.float64)
    kqid = np.ascontiguousarray(kqid, dtype=np.int32)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    tetc = np.asfortranarray(tetc, dtype=np.int32)
    dUl = np.asfortranarray(dUl, dtype=np.float64)
    nbnd, nkp = enk.shape
    nom, nl = dUl.shape
    if nom != omega.shape[0]:
        raise ValueError("dUl must be (nom, nl)")
    ntet = tetc.shape[1]
    nb1, nb2 = ncg + nomx + 1, nbnd - ncg - numin
    kcw = np.zeros((nb1, nb2, nkp, nl), order="F")
    st = _lib(libm).oracle_bz_calcqdepw_par3(_dp(enk), nbnd, nkp, float(ef), _ip(kqid), ncg, nomx, numin, _dp(dUl),
                                             nl, _dp(omega), nom, _ip(tetc), ntet, _dp(kcw), int(nthreads))
    if st < 0:
        raise ValueError("oracle_bz_calcqdepw_par3: bad sizes")
    return kcw


def convw1t(e, f, ef, omega, libm=False):
    """One (tetrahedron, band pair): ``weight[4, nom]``, status, nnod."""
    e = np.ascontiguousarray(e, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float64)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    w = np.zeros((4, omega.shape[0]))
    nn = ctypes.c_longlong(0)
    st = _lib(libm).oracle_convw1t(_dp(e), _dp(f), float(ef), _dp(omega), omega.shape[0], _dp(w), ctypes.byref(nn))
    return w, st, nn.value


def generictetra(corners, e, f, omega, libm=False):
    """generictetra_par on explicit corners [4, 3] (unit-tetrahedron frame)."""
    c = np.ascontiguousarray(corners, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float64)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    w = np.zeros((4, omega.shape[0]))
    info = _lib(libm).oracle_generictetra(_dp(c), _dp(e), _dp(f), _dp(omega), omega.shape[0], _dp(w))
    return w, info


def portable_math(x):
    """(atan(x), log(x)) from the project's portable implementation."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    a = np.empty_like(x)
    lg = np.empty_like(x)
    _lib(False).oracle_portable_math(_dp(x), x.shape[0], _dp(a), _dp(lg))
    return a, lg


class reference_layout:
    """Context manager: inside it the restatement reproduces the reference's
    wtemp(4,2,nom) addressing for 7- and 8-node polyhedra (the first half's
    weights replaced by the second half's, two frequencies earlier, from the
    third frequency on) instead of adding the two halves at every frequency."""

    def __enter__(self):
        for libm in (False, True):
            _lib(libm).oracle_set_reference_layout(1)
        return self

    def __exit__(self, *exc):
        for libm in (False, True):
            _lib(libm).oracle_set_reference_layout(0)
        return False
