"""Independent quadrature of the tetrahedron weight integral (test infrastructure).

A numerical integral of the same integrand, independent of the closed forms
(the reference's and the oracle's): tests/test_oracle_weights.py checks the
oracle against it.

Restates the integrand of ``stweight_numeric`` (for_tetrahedra2.f90:1504-1604,
``iop_omg = 1``): for the unit tetrahedron with energy differences ``de`` at
its corners,

    w_i = ∫_T fw_i(x,y,z) · (−2·E)/(ω² + E²) dx dy dz,
    E = de1 + x(de2−de1) + y(de3−de1) + z(de4−de1),
    fw = [(1−x−y−z), x, y, z],

with nested Gauss–Legendre rules over z ∈ [0,1], y ∈ [0,1−z],
x ∈ [0,1−y−z] (the reference nests gauq_z/gauq_y/gauq_x the same way with
``gauleg`` abscissas).  ``numpy.polynomial.legendre.leggauss`` supplies the
rule; the order is raised well past the reference's 8 so the quadrature
error is far below the tolerance of the comparison.
"""
from __future__ import annotations

import numpy as np


def tet_weights(de, omega, n=48):
    de = np.asarray(de, dtype=float)
    x0, w0 = np.polynomial.legendre.leggauss(n)
    t = 0.5 * (x0 + 1.0)
    wt = 0.5 * w0
    z = t[:, None, None]
    wz = wt[:, None, None]
    y = (1.0 - z) * t[None, :, None]
    wy = (1.0 - z) * wt[None, :, None]
    x = (1.0 - y - z) * t[None, None, :]
    wx = (1.0 - y - z) * wt[None, None, :]
    W = wz * wy * wx
    E = de[0] + x * (de[1] - de[0]) + y * (de[2] - de[0]) + z * (de[3] - de[0])
    fw = [1.0 - x - y - z, x, y, z]
    out = np.zeros((4, len(omega)))
    for io, om in enumerate(omega):
        comm = -2.0 * E / (om * om + E * E)
        for i in range(4):
            out[i, io] = np.sum(W * fw[i] * comm)
    return out
