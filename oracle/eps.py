"""numpy restatement of the χ0 contraction and ε⁻¹ (test infrastructure).

Pinned against the reference's own calc_eps: the reference ships no tests or
golden vectors and its driver (Python 2 with f2py modules) cannot be imported,
so tests/golden/make_calc_eps_golden.py runs the text of calc_eps itself (print
statements rewritten) on seeded inputs and stores its outputs; this
restatement reproduces them exactly for a finite q, q = 0 with head and wings,
and the SVD basis (tests/test_oracle_eps_golden.py).  Known answers
(tests/test_oracle_eps.py) check it as well.

Follows MatrixElements2Band.calc_eps (pygw.py:3039-3297) for a Γ-point or
finite q, with or without the SVD frequency basis:

* k loop (pygw.py:3083-3200): ``minm2 = reshape(minm, (nb1*nb2, matsiz))``,
  ``tmat = minm2.T*coef * kcw[:nb1,:nb2,ik,iom].ravel()`` (coef = −fspin = −2),
  ``eps[:,:,iom] += tmat @ conj(minm2)``, and for q = 0
  ``epsw1[:,iom] += tmat @ pm`` (pygw.py:3192-3195);
* per frequency (pygw.py:3229-3271): ``eps = (eps + epsᴴ)/2``, ``+I``,
  ``inv``, q = 0 head/wings update, ``−I``.

``chi0`` (the accumulated matrix before symmetrisation) is returned as well so
the contraction can be checked on its own.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg


def calc_eps(kcw, minm_k, npb, pm_k=None, head=None, Ul=None, dUl=None):
    """With ``Ul`` (nl, nom) and ``dUl`` (nom, nl) — the SVD frequency basis —
    ``kcw`` holds the par3 weights (nl basis functions) and the flow of
    pygw.py:3043-3045, 3204-3226, 3274-3280 applies: head, wings and ε to
    frequencies with Ul before the inverse, back with dUl after it."""
    nb1, nb2, nkp, nom = kcw.shape
    coef = -2.0
    eps = np.zeros((npb, npb, nom), dtype=complex, order="F")
    epsw1 = np.zeros((npb, nom), dtype=complex)
    iq0 = pm_k is not None
    for ik in range(nkp):
        minm = minm_k(ik)
        minm2 = np.reshape(minm, (nb1 * nb2, npb))
        cminm2 = np.conj(minm2)
        minm2Tc = minm2.T * coef
        pm = pm_k(ik) if iq0 else None
        for iom in range(nom):
            tmat = minm2Tc * kcw[:nb1, :nb2, ik, iom].ravel()
            eps[:, :, iom] += np.matmul(tmat, cminm2)
            if iq0:
                epsw1[:, iom] += np.dot(tmat, pm)
    chi0 = eps.copy(order="F")
    head = None if head is None else np.array(head, dtype=complex)
    if Ul is not None:
        if head is not None:
            head = np.dot(head, Ul)                       # pygw.py:3044-3045
        if iq0:
            epsw1 = np.dot(epsw1, Ul)                     # pygw.py:3206-3208
        eps = np.dot(eps, Ul)                             # pygw.py:3226
        nom = eps.shape[2]
    epsw2 = np.conj(epsw1).copy() if iq0 else None
    Id = np.identity(npb)
    for iom in range(nom):
        eps[:, :, iom] = (eps[:, :, iom] + np.conj(eps[:, :, iom].T)) / 2.0
        eps[:, :, iom] += Id
        eps[:, :, iom] = scipy.linalg.inv(eps[:, :, iom])
        if iq0:
            bw1 = np.dot(eps[:, :, iom], epsw1[:, iom])
            w2b = np.conj(np.dot(eps[:, :, iom], epsw2[:, iom]))
            ww = np.dot(epsw2[:, iom], bw1)
            head[iom] = 1 / (1 + head[iom] - ww)
            epsw1[:, iom] = -head[iom] * bw1[:]
            epsw2[:, iom] = -head[iom] * w2b[:]
            eps[:, :, iom] += head[iom] * np.tensordot(bw1, w2b, axes=0)
            head[iom] -= 1.0
        eps[:, :, iom] -= Id
    if dUl is not None:                                   # pygw.py:3274-3280
        eps = np.dot(eps, dUl)
        if iq0:
            epsw1 = np.dot(epsw1, dUl)
            epsw2 = np.dot(epsw2, dUl)
            head = np.dot(head, dUl)
    if not iq0:
        return eps, None, None, None, chi0
    return eps, epsw1, epsw2, head, chi0
