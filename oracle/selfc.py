"""numpy restatement of the correlation self-energy contraction (test infrastructure).

Pinned against the reference's own code: tests/golden/make_calc_selfc_golden.py
runs the reference's calc_selfc and Compute_selfc_inside (Python) with the
Fortran convolution kernels they call (fnc.f90, no compiler here) executed from
their source text through tests/golden/f90py.py, complex division formed as
compiled Fortran forms it; this restatement reproduces mwm, the energies at
k − q, the iopfreq 4 interpolation and the SVD-branch product, and the
convolutions to the last few bits (numpy's complex division rounds
differently), within 1e-12 (tests/test_oracle_selfc_golden.py).  Known
answers (tests/test_oracle_selfc.py) check the integrals themselves.

Follows MatrixElements2Band.calc_selfc (pygw.py:3299-3412) for one q and the
frequency convolution it calls (mcommon.py:80-131 → fnc.f90:90-177):

* per k (pygw.py:3352-3364): ``minm2 = reshape(minm, (nb1*nb2, matsiz))``,
  ``mw = conj(minm2) @ eps[:,:,iom]``, ``mwm[iom] = wkq * sum(mw * minm2, axis=-1)``
  reshaped (nb1, nb2); for q = 0, for each GW band ie1 the pair
  (ie1, ie1 + ncg_c) gets ``coefs2*head[iom] + coefs1*dot(minm[ie1,ie2,:],
  epsw2[:,iom]) + coefs1*vdot(minm[ie1,ie2,:], epsw1[:,iom])``;
* ``all_fr_convolutions`` (fnc.f90:156-177) with ``fr_convolution2``
  (fnc.f90:90-120): for each (ie1, iom), Σ_ie2 of
  ``eps_om/π · Σ_i (mwm[i]−mwm[iom])·womeg[i]/(ω_i² + eps_om²)
  + mwm[iom]/π · atan(ω_nom/eps_om)`` (the last term only when
  |mwm[iom]| > 1e-16), eps_om = enk[ie2] − i·ω_iom, π = 3.14159265358979 as
  in the Fortran;
* the iopfreq 4 branch (mcommon.py:126-144, spline interpolation onto a
  denser mesh, ``few_fr_convolutions``) and the SVD-basis branch
  (mcommon.py:115-121, ``many_fr_convolutions``, fnc.f90:139-154).

Pinned by known answers (tests/test_oracle_selfc.py): W = c·1 gives
mwm = wkq·c·Σ|M|², and f(Ω) = 1/(Ω² + a²) convolves to
1/(2a(a·sign(e) + e − iω)) in closed form.
"""
from __future__ import annotations

import numpy as np

PI_F = 3.14159265358979      # fnc.f90:71


def mwm_k(minm, eps, wkq, q0=None):
    """mwm[nom, nb1, nb2] for one k.  ``eps`` is (N, N, nom) (ε⁻¹ − 1);
    ``q0`` = (head, epsw1, epsw2, coefs1, coefs2, ncg_c, ibgw) for q = 0,
    with the GW band window starting at ibgw (ie1 = ibgw + row)."""
    nb1, nb2, matsiz = minm.shape
    nom = eps.shape[2]
    minm2 = np.reshape(minm, (nb1 * nb2, matsiz))
    cminm2 = np.conj(minm2)
    out = np.zeros((nom, nb1, nb2), dtype=complex)
    for iom in range(nom):
        mw = np.matmul(cminm2, eps[:, :, iom])
        out[iom] = np.reshape(wkq * np.sum(mw * minm2, axis=-1), (nb1, nb2))
        if q0 is not None:
            head, epsw1, epsw2, coefs1, coefs2, ncg_c, ibgw = q0
            for r in range(nb1):
                ie2 = ibgw + r + ncg_c
                d2 = (coefs2 * head[iom] + coefs1 * np.dot(minm[r, ie2, :], epsw2[:, iom])
                      + coefs1 * np.vdot(minm[r, ie2, :], epsw1[:, iom]))
                out[iom, r, ie2] += d2
    return out


def fr_convolution2(enk, mwm, mwm_iom, omega, omega_iom, womeg):
    eps_om = complex(enk, -omega_iom)
    eps_om2 = eps_om * eps_om
    sc0 = 0j
    for i in range(len(omega)):
        sc0 = sc0 + (mwm[i] - mwm_iom) * womeg[i] / (omega[i] ** 2 + eps_om2)
    res = eps_om * sc0 / PI_F
    if abs(mwm_iom) > 1e-16:
        res = res + mwm_iom / PI_F * np.arctan(omega[-1] / eps_om)
    return res


def all_fr_convolutions(enk, mwm, omega, womeg):
    """sc_p[nb1, nom] from mwm[nom, nb1, nb2] and the energies enk[nb2] (at k−q, core first)."""
    nom, nb1, nb2 = mwm.shape
    sc = np.zeros((nb1, nom), dtype=complex)
    for ie1 in range(nb1):
        for iom in range(nom):
            s = 0j
            for ie2 in range(nb2):
                s = s + fr_convolution2(enk[ie2], mwm[:, ie1, ie2], mwm[iom, ie1, ie2], omega, omega[iom], womeg)
            sc[ie1, iom] = s
    return sc


def interp_fr_convolutions(enk, mwm, omega, omega_precise, womeg_precise):
    """iopfreq 4 branch of Compute_selfc_inside (mcommon.py:126-144): per
    (ie1, ie2) a cubic spline of mwm·(ω²+1) (natural at the first point,
    zero slope at the last, extrapolating) evaluated on the dense mesh, the
    imaginary part only where its mean magnitude exceeds 1e-10; then
    few_fr_convolutions (fnc.f90:179-193) with mwm at the coarse ω_iom."""
    from scipy import interpolate
    nom, nb1, nb2 = mwm.shape
    sc = np.zeros((nb1, nom), dtype=complex)
    fa = omega ** 2 + 1.0
    fp = omega_precise ** 2 + 1.0
    bc = ((2, 0.0), (1, 0.0))
    for ie1 in range(nb1):
        mwmp = np.zeros((nb2, len(omega_precise)), dtype=complex)
        for ie2 in range(nb2):
            sr = interpolate.CubicSpline(omega, fa * mwm[:, ie1, ie2].real, bc_type=bc, extrapolate=True)
            if np.sum(np.abs(mwm[:, ie1, ie2].imag)) / nom > 1e-10:
                si = interpolate.CubicSpline(omega, fa * mwm[:, ie1, ie2].imag, bc_type=bc, extrapolate=True)
                mwmp[ie2, :] = (sr(omega_precise) + si(omega_precise) * 1j) / fp
            else:
                mwmp[ie2, :] = sr(omega_precise) / fp
        for iom in range(nom):
            s = 0j
            for ie2 in range(nb2):
                s = s + fr_convolution2(enk[ie2], mwmp[ie2, :], mwm[iom, ie1, ie2], omega_precise, omega[iom],
                                        womeg_precise)
            sc[ie1, iom] = s
    return sc


def many_fr_convolutions(enk, Ul, omega, womeg):
    """Cnl[nl, nb2, nom] (fnc.f90:139-154): the convolution of every SVD basis function."""
    nl, nom = Ul.shape
    nb2 = len(enk)
    cnl = np.zeros((nl, nb2, nom), dtype=complex)
    for il in range(nl):
        for iom in range(nom):
            for ie2 in range(nb2):
                cnl[il, ie2, iom] = fr_convolution2(enk[ie2], Ul[il, :], Ul[il, iom], omega, omega[iom], womeg)
    return cnl


def svd_fr_convolutions(enk, mwm, Ul, omega, womeg):
    """SVD-basis branch (mcommon.py:115-121): mwm[nl, nb1, nb2] in the basis;
    sc_p = mwm2 · reshape(Cnl, (nl·nb2, nom)), mwm2[ie1] = ravel(mwm[:, ie1, :])."""
    nl, nb1, nb2 = mwm.shape
    nom = Ul.shape[1]
    cnl = np.reshape(many_fr_convolutions(enk, Ul, omega, womeg), (nl * nb2, nom))
    mwm2 = np.zeros((nb1, nl * nb2), dtype=complex)
    for ie1 in range(nb1):
        mwm2[ie1, :] = np.reshape(mwm[:, ie1, :], nl * nb2)
    return np.dot(mwm2, cnl)
