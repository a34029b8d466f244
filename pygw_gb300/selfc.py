"""Correlation self-energy on the GPU — the GB300 branch of ``MatrixElements2Band.calc_selfc``.

``mwm`` runs the contraction of pygw.py:3352-3364 for a chunk of k-points
(FP64, or the split-precision tensor-core GEMM), ``mwm_q0`` its q = 0 head
and wing terms, ``convolution`` the Matsubara convolution of
Compute_selfc_inside (mcommon.py:80-165) in its three forms: the plain
``all_fr_convolutions``, the iopfreq 4 spline interpolation onto
``fr.omega_precise``, and the SVD basis.  ``calc_selfc`` strings them
together with the reference's signature (pygw.py:3299) and returns
``sc_p[nirkp, nbgw − ibgw, nom]``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from . import eps as _eps
from .device import ptr, require_cuda, stream_handle, to_device, workspace

WORK_BUDGET = 8 << 30        # bytes of digit/tile workspace for the split-precision contraction


def _eps_device(eps):
    """ε⁻¹ − 1 as a CUDA complex128 tensor [nom][N][N] whose storage is the
    Fortran order of (N, N, nom) — the layout EpsResult.eps holds."""
    if isinstance(eps, torch.Tensor):
        return eps.contiguous()
    if hasattr(eps, "eps"):                  # EpsResult
        return eps.eps
    a = np.asarray(eps, dtype=np.complex128)
    return to_device(a.transpose(2, 1, 0), torch.complex128)


def _vec_device(a, nom, n=None):
    """head [nom] or wings (N, nom) (reference layouts) → CUDA [nom] / [nom][N]."""
    if a is None or isinstance(a, torch.Tensor):
        return a
    a = np.asarray(a, dtype=np.complex128)
    return to_device(a.T if a.ndim == 2 else a, torch.complex128)


def mixed_k_chunk(P, npb, nom, budget=None):
    """(k-chunk, ω batch) whose split-precision workspace stays within the budget."""
    budget = WORK_BUDGET if budget is None else budget
    per_row = 56 * npb + 16 * npb          # A digits and the float-pair copy of M + one frequency of tiles
    nk = max(1, int(budget // 2 // max(1, per_row * P)))
    lib = _lib.load()
    nb = nom
    while nb > 1 and lib.pg_selfc_mwm_workspace(nk, P, npb, nb, 1) > budget:
        nb = (nb + 1) // 2
    return nk, nb


def mwm(minm, eps, nb1, nb2, wkq, precision=None, omega_batch=None, stream=None, work=None, out=None, status=None):
    """mwm[k][ω][p] (torch complex128, p = ib1·nb2 + ib2) for the k-points of
    ``minm`` ([nk][nb1][nb2][N] or [nk][P][N], numpy or torch) and the
    frequencies of ``eps`` (ε⁻¹ − 1, see _eps_device)."""
    require_cuda()
    lib = _lib.load()
    precision = precision or _eps.PRECISION
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
    W = _eps_device(eps)
    nom, N = W.shape[0], W.shape[1]
    P = nb1 * nb2
    M = to_device(minm, torch.complex128).reshape(-1, P, N)
    nk = M.shape[0]
    if out is None:
        out = torch.empty((nk, nom, P), dtype=torch.complex128, device="cuda")
    mixed = 1 if precision == "mixed" else 0
    nb = omega_batch or (mixed_k_chunk(P, N, nom)[1] if mixed else nom)
    if mixed and work is None:
        work = workspace(lib.pg_selfc_mwm_workspace(nk, P, N, nb, 1))
    st = status if status is not None else torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.pg_selfc_mwm(M.data_ptr(), nk, P, N, W.data_ptr(), nom, float(wkq), out.data_ptr(), mixed, nb,
                          ptr(work), 0 if work is None else work.numel(), st.data_ptr(), stream_handle(stream))
    _lib.check(rc, "pg_selfc_mwm")
    if status is None and mixed:
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
        if int(st.item()) != 0:
            raise _lib.PygwError(f"pg_selfc_mwm: device status {int(st.item()):#x}")
    return out


def mwm_q0(out, minm, nb1, nb2, off, head, epsw1, epsw2, coefs1, coefs2, stream=None):
    """Adds the q = 0 terms (pygw.py:3358-3363) to ``out`` in place; off = ibgw + ncg_c."""
    lib = _lib.load()
    nk, nom, P = out.shape
    N = epsw1.shape[-1] if isinstance(epsw1, torch.Tensor) else np.asarray(epsw1).shape[0]
    M = to_device(minm, torch.complex128).reshape(nk, P, N)
    h = to_device(np.asarray(head, dtype=np.complex128), torch.complex128) if not isinstance(head, torch.Tensor) \
        else head
    w1, w2 = _vec_device(epsw1, nom), _vec_device(epsw2, nom)
    rc = lib.pg_selfc_mwm_q0(M.data_ptr(), nk, nb1, nb2, N, int(off), nom, h.data_ptr(), w1.data_ptr(),
                             w2.data_ptr(), float(coefs1), float(coefs2), out.data_ptr(), stream_handle(stream))
    _lib.check(rc, "pg_selfc_mwm_q0")
    return out


def spline_matrix(omega, omega_dense):
    """S[j][i]: the cubic spline through (ω_i, e_i) (second derivative 0 at the
    first point, slope 0 at the last, extrapolating — the boundary conditions of
    mcommon.py:135) at ωd_j.  The spline is linear in its data, so
    spline(y)(ωd) = S·y for every column y."""
    from scipy import interpolate
    omega = np.asarray(omega, dtype=np.float64)
    n = omega.shape[0]
    z = np.zeros(n)          # one boundary value per column of the data
    sp = interpolate.CubicSpline(omega, np.eye(n), axis=0, bc_type=((2, z), (1, z)), extrapolate=True)
    return np.ascontiguousarray(sp(np.asarray(omega_dense, dtype=np.float64)))


def convolution(mwm_d, enk, omega, womeg, nb1, nb2, dense=None, Ul=None, stream=None):
    """sc[k][ie1][iom] (torch complex128) from mwm[k][·][p] and enk[k][nb2].
    dense = (omega_precise, womeg_precise) selects the iopfreq 4 branch;
    Ul (nl, nom) the SVD basis (mwm then has nl entries per k)."""
    require_cuda()
    lib = _lib.load()
    nk = mwm_d.shape[0]
    nom = len(omega)
    om = to_device(np.asarray(omega, dtype=np.float64))
    wom = to_device(np.asarray(womeg, dtype=np.float64))
    e = to_device(np.asarray(enk, dtype=np.float64).reshape(nk, nb2))
    sc = torch.empty((nk, nb1, nom), dtype=torch.complex128, device="cuda")
    sh = stream_handle(stream)
    if Ul is not None:
        U = to_device(np.asarray(Ul, dtype=np.complex128))
        nl = U.shape[0]
        if mwm_d.shape[1] != nl or U.shape[1] != nom:
            raise ValueError("SVD convolution: mwm must hold nl basis entries and Ul be (nl, nom)")
        work = workspace(lib.pg_selfc_convolution_workspace(nk, nb1, nb2, nom, 0, nl))
        rc = lib.pg_selfc_convolution_svd(mwm_d.data_ptr(), nk, nb1, nb2, nl, nom, e.data_ptr(), U.data_ptr(),
                                          om.data_ptr(), wom.data_ptr(), work.data_ptr(), work.numel(),
                                          sc.data_ptr(), sh)
        _lib.check(rc, "pg_selfc_convolution_svd")
        return sc
    if dense is None or len(dense[0]) == nom:
        # the reference takes the plain branch whenever the dense mesh has nom points (mcommon.py:123)
        rc = lib.pg_selfc_convolution(mwm_d.data_ptr(), nk, nb1, nb2, nom, e.data_ptr(), om.data_ptr(),
                                      wom.data_ptr(), 0, None, None, None, None, 0, sc.data_ptr(), sh)
        _lib.check(rc, "pg_selfc_convolution")
        return sc
    omd = np.asarray(dense[0], dtype=np.float64)
    S = to_device(spline_matrix(omega, omd))
    omd_d = to_device(omd)
    womd = to_device(np.asarray(dense[1], dtype=np.float64))
    nd = omd.shape[0]
    work = workspace(lib.pg_selfc_convolution_workspace(nk, nb1, nb2, nom, nd, 0))
    rc = lib.pg_selfc_convolution(mwm_d.data_ptr(), nk, nb1, nb2, nom, e.data_ptr(), om.data_ptr(), None, nd,
                                  omd_d.data_ptr(), womd.data_ptr(), S.data_ptr(), work.data_ptr(), work.numel(),
                                  sc.data_ptr(), sh)
    _lib.check(rc, "pg_selfc_convolution")
    return sc


def _selfc_enk(bands, ncg_c, core, jrk, nb2, isp=0):
    """Energies at k−q, core first (mcommon.py:103-108)."""
    enk = np.zeros(nb2)
    for icg in range(ncg_c):
        iat, idf, ic = core.corind[icg, :3]
        enk[icg] = core.eig_core[isp][iat][ic]
    enk[ncg_c:nb2] = bands[jrk, :(nb2 - ncg_c)]
    return enk


def calc_selfc(me, iq, eps, epsw1, epsw2, head, strc, in1, latgen, kqm, ks, radf, pw, pb, core, kw, fr, ddir, dUl,
               Ul, fout, PRINT=True, precision=None, k_chunk=None):
    """The body of MatrixElements2Band.calc_selfc (pygw.py:3299-3412) for the
    object ``me`` (its ``calc_minm``, ``singc1``, ``singc2``).  Matrix
    elements are built per irreducible k on the host, as in the reference, and
    contracted on the GPU a chunk of k-points at a time."""
    require_cuda()
    isp = 0
    wkq = 1.0 / len(kqm.qlist)
    coefs1 = coefs2 = 0.0
    if iq == 0:
        coefs2 = me.singc2 * 4 * np.pi / latgen.Vol
        coefs1 = me.singc1 * np.sqrt(4 * np.pi / latgen.Vol)
    W = _eps_device(eps)
    nom_nil, N = W.shape[0], W.shape[1]
    nirkp = len(kqm.weight)
    nb1 = ks.nbgw - ks.ibgw
    nb2 = ks.nbands_c
    P = nb1 * nb2
    nom = len(fr.omega)
    precision = precision or _eps.PRECISION
    if k_chunk is None:
        k_chunk = mixed_k_chunk(P, N, nom_nil)[0] if precision == "mixed" else max(1, int((2 << 30) // (16 * P * N)))
    band_limits = (ks.ibgw, ks.nbgw, 0, ks.nbands_c - ks.ncg_c, 0, ks.ncg_c)
    dense = None
    if getattr(fr, "iopfreq", None) == 4 and hasattr(fr, "omega_precise"):
        dense = (fr.omega_precise, fr.womeg_precise)
    q0 = None
    if iq == 0:
        q0 = (_vec_device(head, nom_nil), _vec_device(epsw1, nom_nil), _vec_device(epsw2, nom_nil))
    sc_p = np.zeros((nirkp, nb1, nom), dtype=complex)
    for k0 in range(0, nirkp, k_chunk):
        ks_ = range(k0, min(nirkp, k0 + k_chunk))
        mins, enks = [], []
        for irk in ks_:
            ik = kqm.k_ind[irk]
            jk = kqm.kqid[ik, iq]
            jrk = kqm.kii_ind[jk]
            minm0, minc0 = me.calc_minm(ik, iq, band_limits, "selfe")
            m = minm0 if minc0 is None else np.concatenate((minc0, minm0), axis=1)
            if m.shape[:2] != (nb1, nb2):
                raise ValueError(f"calc_minm returned {m.shape[:2]}, expected {(nb1, nb2)}")
            mins.append(np.ascontiguousarray(m, dtype=np.complex128))
            enks.append(_selfc_enk(ks.Ebnd[isp], ks.ncg_c, core, jrk, nb2, isp))
        M = to_device(np.stack(mins))
        mw = mwm(M, W, nb1, nb2, wkq, precision=precision)
        if iq == 0:
            mwm_q0(mw, M, nb1, nb2, ks.ibgw + ks.ncg_c, q0[0], q0[1], q0[2], coefs1, coefs2)
        sc = convolution(mw, np.stack(enks), fr.omega, fr.womeg, nb1, nb2, dense=dense, Ul=Ul)
        sc_p[k0:k0 + len(ks_)] = sc.cpu().numpy()
    if PRINT and fout is not None:
        for irk in range(nirkp):
            for ie1 in range(nb1):
                print('dSigc[iq=%3d,irk=%3d,ie=%3d,iom=%3d]=%16.12f%16.12f' %
                      (iq, irk, ie1 + ks.ibgw, 0, sc_p[irk, ie1, 0].real, sc_p[irk, ie1, 0].imag), file=fout)
    return sc_p
