"""SVD frequency basis (PyGW's ``iopfreq = 5``): basis construction, the
par3 weights and the basis changes around ε⁻¹.

* ``tan_mesh`` / ``svd_functions`` build the basis the reference builds in
  ``Give2TanMesh`` (mcommon.py:13-31) and ``svd_functions`` (pygw.py:3478-3501):
  the bosonic kernel K(iω_n, ω) = (ω dω/π)·√dω_n / (ω² + ω_n²) between the
  Matsubara points (both signs) and a real-axis tan mesh is decomposed, the
  singular vectors above ``svd_cutoff`` are kept, ``Ul`` (nl, nom) maps basis
  coefficients to frequencies and ``dUl`` (nom, nl) projects back
  (``Ul @ dUl = I``).  Host-side setup, done once.
* ``bz_calcqdepw_par3`` is the drop-in for ``ft.bz_calcqdepw_par3``
  (pygw.py:3441): ``pg_bz_calcqdepw_par3`` on the GPU.
* ``to_basis`` applies a real basis matrix along the leading (frequency /
  basis) index of device arrays (``pg_basis_change``).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg
import scipy.optimize
import torch

from . import _lib
from .device import ptr, require_cuda, stream_handle, to_device, workspace
from .polarization import STAT_NAMES, STATUS_BITS, WeightsResult


def tan_mesh(x0, L, Nw):
    """2·Nw points ω = w·tan(x) on (−L, L) with the smallest |ω| ≈ x0, and their
    weights dω (a tangent mesh dense near 0).  (d, w) solve L = w/tan(d) and
    x0 = w·tan(π/(2Nw) − d/Nw)."""
    tnw = np.tan(np.pi / (2 * Nw))
    if x0 > L * 0.25 * Nw * tnw ** 2:
        x0 = L * 0.25 * Nw * tnw ** 2 - 1e-15
    xi = x0 / L
    d0 = Nw / 2.0 * (tnw - np.sqrt(tnw ** 2 - 4 * xi / Nw))

    def eqs(v):
        d, w = v
        return [L - w / np.tan(d), x0 - w * np.tan(np.pi / (2 * Nw) - d / Nw)]

    d, w = scipy.optimize.root(eqs, [d0, L * d0]).x
    x = np.linspace(0.0, 1.0, 2 * Nw) * (np.pi - 2 * d) - np.pi / 2 + d
    return w * np.tan(x), (w * (np.pi - 2 * d) / (2.0 * Nw)) / np.cos(x) ** 2


def svd_functions(iomega, wiomeg, om_min, om_max, om_nom, svd_cutoff):
    """(Ul[nl, nom], dUl[nom, nl]) of the bosonic Matsubara kernel for the
    positive Matsubara points ``iomega`` with weights ``wiomeg``."""
    om, dom = tan_mesh(om_min, om_max, om_nom)
    iw = np.concatenate([-iomega[::-1], iomega])
    dw = np.concatenate([wiomeg[::-1], wiomeg])
    K = (om * dom / np.pi)[None, :] * np.sqrt(dw)[:, None] / (om[None, :] ** 2 + iw[:, None] ** 2)
    u, s, _ = scipy.linalg.svd(K, full_matrices=True)          # the reference's routine (pygw.py:3490)
    small = np.where(s < svd_cutoff)[0]
    n = int(small[0]) if len(small) else len(s)
    Ul = u[:, :n].T / np.sqrt(dw)[None, :]
    h = len(iw) // 2
    dUl = (Ul[:, h:] * dw[h:] * 2.0).T          # positive frequencies only, hence the factor 2
    return Ul[:, h:].copy(), dUl.copy()


def weights_device_par3(enk, ef, kqid, ncg, nomx, numin, dUl, omega, tetc, stream=None):
    """par3 weights left on the GPU: ``WeightsResult`` with shape (nb1, nb2, nkp, nl)."""
    require_cuda()
    lib = _lib.load()
    enk = np.asarray(enk, dtype=np.float64)
    nbnd, nkp = enk.shape
    tetc = np.asarray(tetc)
    ntet = tetc.shape[1]
    dUl = np.asarray(dUl, dtype=np.float64)
    nom, nl = dUl.shape
    enk_d = to_device(enk.T, torch.float64)
    tetc_d = to_device(tetc.astype(np.int32).T, torch.int32)
    kqid_d = to_device(np.asarray(kqid, dtype=np.int32), torch.int32)
    om_d = to_device(np.asarray(omega, dtype=np.float64), torch.float64)
    du_d = to_device(dUl.T, torch.float64)                       # (nom, nl) Fortran = [nl][nom] C order
    nb1, nb2 = ncg + nomx + 1, nbnd - ncg - numin
    kcw = torch.empty((nl, nkp, nb2, nb1), dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    counters = torch.zeros(len(STAT_NAMES), dtype=torch.int64, device="cuda")
    work = workspace(lib.pg_bz_calcqdepw_par3_workspace(nbnd, nkp, ncg, nomx, numin, nom, ntet, nl))
    rc = lib.pg_bz_calcqdepw_par3(ptr(enk_d), nbnd, nkp, float(ef), ptr(kqid_d), ncg, nomx, numin, ptr(du_d), nl,
                                  ptr(om_d), nom, ptr(tetc_d), ntet, ptr(kcw), ptr(work), work.numel(), ptr(status),
                                  ptr(counters), stream_handle(stream))
    _lib.check(rc, "pg_bz_calcqdepw_par3")
    return WeightsResult(kcw, status, counters, (nb1, nb2, nkp, nl))


def bz_calcqdepw_par3(enk, ef, kqid, ncg, nomx, numin, dUl, omega, tetc):
    """Same call and result as the reference's ``ft.bz_calcqdepw_par3`` (pygw.py:3441)."""
    r = weights_device_par3(enk, ef, kqid, ncg, nomx, numin, dUl, omega, tetc)
    torch.cuda.synchronize()
    st = r.status
    if st:
        bits = [v for b, v in STATUS_BITS.items() if st & b]
        raise _lib.PygwError(f"bz_calcqdepw_par3: reference error condition(s) {bits}")
    return r.numpy()


def to_basis(x, U, stream=None):
    """y[j, ...] = Σ_i x[i, ...]·U[i, j] for a complex CUDA tensor x whose leading
    index is a frequency or basis index; U real (nin, nout)."""
    lib = _lib.load()
    U = np.asarray(U, dtype=np.float64)
    nin, nout = U.shape
    if x.shape[0] != nin:
        raise ValueError("leading dimension does not match the basis matrix")
    x = x.contiguous()
    nelem = x.numel() // nin
    y = torch.empty((nout,) + tuple(x.shape[1:]), dtype=torch.complex128, device="cuda")
    u_d = to_device(U.T, torch.float64)                           # Fortran (nin, nout)
    rc = lib.pg_basis_change(ptr(x), nin, ptr(y), nout, ptr(u_d), int(nelem), stream_handle(stream))
    _lib.check(rc, "pg_basis_change")
    return y
