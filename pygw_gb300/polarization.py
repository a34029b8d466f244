"""Tetrahedron polarization weights — the GB300 branch of PyGW's ``Polarization_weights``.

``Polarization_weights`` keeps the reference's signature (pygw.py:3416) and
``bz_calcqdepw_par2`` the f2py call's (pygw.py:3443, for_tetrahedra.f90:390):
Fortran-ordered numpy arrays in, ``kcw[ncg+nomx+1, nbnd-ncg-numin, nkp, nom]``
out.  ``weights_device`` is the same computation leaving ``kcw`` on the GPU
for the χ0 contraction.

The reference has no ``if FORT`` switch at this call site; the switch is
added here in the form the reference uses elsewhere (kqmesh.py:363-373),
widened to three values: ``'python'`` and ``'fortran'`` name the reference's
own implementations (not part of this package), ``'gb300'`` is this one.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .device import ptr, require_cuda, stream_handle, to_device, workspace

FORT = "gb300"
STAT_NAMES = (["calls"] + [f"nnod{i}" for i in range(9)] + [f"equiv{i}" for i in (4, 6, 8, 10, 16)]
              + ["taylor", "exact", "zero_vol", "big_weight_warn", "big_weight_zeroed"])
STATUS_BITS = {1: "nnod>8", 2: "sorteq", 4: "sortnodes", 8: "relnodes", 16: "equiv_flag", 32: "undefined",
               64: "non-finite"}


class WeightsResult:
    """Device ``kcw`` plus the kernel's status word and counters."""

    def __init__(self, kcw, status, counters, shape):
        self.kcw = kcw              # torch CUDA float64, storage = F order of `shape`
        self.shape = shape          # (nb1, nb2, nkp, nom)
        self._status = status
        self._counters = counters

    @property
    def status(self) -> int:
        return int(self._status.item())

    @property
    def counters(self) -> dict:
        return dict(zip(STAT_NAMES, self._counters.cpu().tolist()))

    def numpy(self):
        """``kcw`` as the reference returns it (Fortran-ordered float64)."""
        return self.kcw.cpu().numpy().transpose(3, 2, 1, 0)


def weights_device(enk, ef, kqid, ncg, nomx, numin, omega, tetc, nom_chunk=0, stream=None, work=None):
    """Compute ``kcw`` on the GPU; arguments as in ``bz_calcqdepw_par2``.

    ``enk`` [nbnd, nkp] and ``tetc`` [4, ntet] may be numpy (any order) or
    tensors already laid out as the C-ABI expects (enk as [nkp][nbnd], tetc as
    [ntet][4]); CPU tensors (pinned for asynchronous copies) are copied to the
    device on the current stream.
    """
    require_cuda()
    lib = _lib.load()
    if isinstance(enk, np.ndarray):
        nbnd, nkp = enk.shape
        enk_d = to_device(np.asarray(enk, dtype=np.float64).T, torch.float64)   # [nkp][nbnd]
    else:
        nkp, nbnd = enk.shape
        enk_d = to_device(enk, torch.float64)
    if isinstance(tetc, np.ndarray):
        ntet = tetc.shape[1]
        tetc_d = to_device(np.asarray(tetc, dtype=np.int32).T, torch.int32)    # [ntet][4]
    else:
        ntet = tetc.shape[0]
        tetc_d = to_device(tetc, torch.int32)
    kqid_d = to_device(np.asarray(kqid, dtype=np.int32) if isinstance(kqid, np.ndarray) else kqid, torch.int32)
    om_d = to_device(np.asarray(omega, dtype=np.float64) if isinstance(omega, np.ndarray) else omega, torch.float64)
    nom = int(om_d.shape[0])
    nb1, nb2 = ncg + nomx + 1, nbnd - ncg - numin
    if nb1 <= 0 or nb2 <= 0:
        raise ValueError("empty band window")
    kcw = torch.empty((nom, nkp, nb2, nb1), dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    counters = torch.zeros(len(STAT_NAMES), dtype=torch.int64, device="cuda")
    wb = lib.pg_bz_calcqdepw_par2_workspace(nbnd, nkp, ncg, nomx, numin, nom, ntet, int(nom_chunk))
    if work is None or work.numel() < wb:
        work = workspace(wb)
    rc = lib.pg_bz_calcqdepw_par2(ptr(enk_d), nbnd, nkp, float(ef), ptr(kqid_d), ncg, nomx, numin, ptr(om_d), nom,
                                  ptr(tetc_d), ntet, ptr(kcw), ptr(work), work.numel(), int(nom_chunk),
                                  ptr(status), ptr(counters), stream_handle(stream))
    _lib.check(rc, "pg_bz_calcqdepw_par2")
    return WeightsResult(kcw, status, counters, (nb1, nb2, nkp, nom))


class reference_layout:
    """Context manager: weights computed inside it reproduce the reference's
    addressing of its wtemp(4,2,nom) array for 7- and 8-node polyhedra
    (for_tetrahedra3.f90:36, 100-120), equal to the reference's statements at
    every entry; outside it the two halves are added at every frequency
    (``pg_set_weights_reference_layout``)."""

    def __enter__(self):
        lib = _lib.load()
        self.prev = lib.pg_weights_reference_layout()
        _lib.check(lib.pg_set_weights_reference_layout(1), "pg_set_weights_reference_layout")
        return self

    def __exit__(self, *exc):
        _lib.load().pg_set_weights_reference_layout(self.prev)
        return False


def bz_calcqdepw_par2(enk, ef, kqid, ncg, nomx, numin, omega, tetc):
    """Same call and result as the reference's ``ft.bz_calcqdepw_par2`` (pygw.py:3443)."""
    r = weights_device(enk, ef, kqid, ncg, nomx, numin, omega, tetc)
    torch.cuda.synchronize()
    st = r.status
    if st:
        bits = [v for b, v in STATUS_BITS.items() if st & b]
        raise _lib.PygwError(f"bz_calcqdepw_par2: reference error condition(s) {bits}")
    return r.numpy()


def assemble_enk(ks, kqm, core, isp=0):
    """``enk[nbnd, nkp]`` = core energies ‖ KS bands up to nbmaxpol (pygw.py:3418-3426)."""
    ankp = len(kqm.kii_ind)
    nbnd = ks.ncg_p + ks.nbmaxpol
    enk = np.zeros((nbnd, ankp), order="F")
    for icg in range(ks.ncg_p):
        iat, idf, ic = core.corind[icg][0:3]
        enk[icg, :] = core.eig_core[isp][iat][ic]
    for ik in range(ankp):
        irk = kqm.kii_ind[ik]
        enk[ks.ncg_p:(ks.ncg_p + ks.nbmaxpol), ik] = ks.Ebnd[isp, irk, :ks.nbmaxpol]
    return enk


def Polarization_weights(iq, ks, kqm, core, fr, iop_bzintq, sgnfrq, dUl, fout, isp=0):
    """Drop-in for pygw.py:3416 (GB300 branch).  Returns ``kcw`` as a numpy array."""
    if FORT != "gb300":
        raise RuntimeError("pygw_gb300 implements only the 'gb300' branch of the FORT switch")
    nomx, numin = ks.nomax_numin
    enk = assemble_enk(ks, kqm, core, isp)
    if dUl is not None:
        from .svd import bz_calcqdepw_par3
        return bz_calcqdepw_par3(enk, ks.EF, kqm.kqid[:, iq], ks.ncg_p, nomx, numin, dUl, fr.omega, kqm.tetc)
    return bz_calcqdepw_par2(enk, ks.EF, kqm.kqid[:, iq], ks.ncg_p, nomx, numin, fr.omega, kqm.tetc)
