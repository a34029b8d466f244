"""ctypes binding of ``libpygw_gb300.so`` (the C-ABI declared in include/pygw_gb300.h).

There is no fallback: if the library is missing or fails to load, importing
the GPU path raises.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

c_int, c_size_t, c_double, c_void_p = ctypes.c_int, ctypes.c_size_t, ctypes.c_double, ctypes.c_void_p
c_longlong = ctypes.c_longlong
c_uint_p = ctypes.POINTER(ctypes.c_uint)
c_ull_p = ctypes.POINTER(ctypes.c_ulonglong)

# name -> (restype, argtypes)
SIGNATURES = {
    "pg_bz_calcqdepw_par2_workspace": (c_size_t, [c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_int]),
    "pg_bz_calcqdepw_par2": (c_int, [c_void_p, c_int, c_int, c_double, c_void_p, c_int, c_int, c_int, c_void_p,
                                     c_int, c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_int, c_void_p,
                                     c_void_p, c_void_p]),
    "pg_bz_calcqdepw_par2_noalloc_capacity": (c_size_t, []),
    "pg_bz_calcqdepw_par2_noalloc": (c_int, [c_void_p, c_int, c_int, c_double, c_void_p, c_int, c_int, c_int,
                                             c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                             c_void_p]),
    "pg_chi0_accumulate_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_int, c_int, c_int,
                                       c_double, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pg_chi0_mirror_f64": (c_int, [c_void_p, c_int, c_int, c_void_p]),
    "pg_eps_inverse_f64_workspace": (c_size_t, [c_int, c_int]),
    "pg_chi0_mixed_workspace": (c_size_t, [c_int, c_int, c_int, c_int, c_int, c_int]),
    "pg_chi0_mixed": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_int, c_double, c_void_p, c_void_p,
                              c_size_t, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "pg_eps_inverse_mixed_workspace": (c_size_t, [c_int, c_int, c_int]),
    "pg_eps_inverse_mixed": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_int,
                                     c_int, c_void_p, c_void_p]),
    "pg_chi0_mixed_accumulate": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_longlong, c_void_p, c_int,
                                         c_int, c_int, c_int, c_int, c_double, c_void_p, c_int, c_void_p, c_size_t,
                                         c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "pg_synth_minm": (c_int, [c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_int, c_void_p,
                              c_void_p, c_longlong, c_void_p, c_int, ctypes.c_ulonglong, c_void_p, c_void_p]),
    "pg_bz_calcqdepw_par3_workspace": (c_size_t, [c_int] * 8),
    "pg_bz_calcqdepw_par3": (c_int, [c_void_p, c_int, c_int, c_double, c_void_p, c_int, c_int, c_int, c_void_p, c_int,
                                     c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_void_p,
                                     c_void_p, c_void_p]),
    "pg_basis_change": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_longlong, c_void_p]),
    "pg_chi0_mixed_layout": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
    "pg_wings_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_int, c_int, c_int, c_double,
                             c_void_p, c_void_p, c_void_p]),
    "pg_selfc_mwm_workspace": (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    "pg_selfc_mwm": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_double, c_void_p, c_int, c_int,
                             c_void_p, c_size_t, c_void_p, c_void_p]),
    "pg_selfc_mwm_q0": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                c_double, c_double, c_void_p, c_void_p]),
    "pg_selfc_convolution_workspace": (c_size_t, [c_int] * 6),
    "pg_selfc_convolution": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int,
                                     c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p]),
    "pg_selfc_convolution_svd": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_size_t, c_void_p, c_void_p]),
    "pg_launch_count": (ctypes.c_ulonglong, []),
    "pg_set_wait_limit_ns": (None, [ctypes.c_ulonglong]),
    "pg_wait_limit_ns": (ctypes.c_ulonglong, []),
    "pg_set_chi0_prep_batch": (c_int, [c_int]),
    "pg_chi0_prep_batch": (c_int, []),
    "pg_set_weights_reference_layout": (c_int, [c_int]),
    "pg_weights_reference_layout": (c_int, []),
    "pg_eps_inverse_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                                   c_void_p]),
}

ERRORS = {-1: "invalid argument", -2: "workspace too small", -3: "CUDA launch failed", -4: "request exceeds capacity"}

_lib = None


class PygwError(RuntimeError):
    pass


def load(path: str | None = None):
    """Load the library (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        from .build import build
        build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str):
    if rc != 0:
        raise PygwError(f"{what}: {ERRORS.get(rc, rc)}")
