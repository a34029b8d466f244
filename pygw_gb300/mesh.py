"""Γ-centred k/q mesh and its tetrahedra, restating PyGW's ``KQmesh.tetra``.

Only the parts the polarization path consumes are built here:

* ``tetc[4, 6*nkp]`` (Fortran order, 0-based k indices) — six tetrahedra per
  cube, all sharing the shortest main diagonal of the cube
  (kqmesh.py:195-257; the diagonal choice ``mnd`` is kqmesh.py:203-239);
* ``kqid[nkp, nkp]`` — index of k−q for every (k, q) (for_kpts.f90:21-45,
  kqmesh.py:363-373);
* ``k2indx`` / ``indx2k`` (for_kpts.f90:1-18).

Symmetry reduction (irreducible k points, ``atet``/``wtet``) needs a crystal
and is not part of the hot path; every k of the full mesh is its own
irreducible point (``kii_ind = arange(nkp)``).
"""
from __future__ import annotations

import itertools

import numpy as np

# The six tetrahedra of the unit cube around the (0,0,0)-(1,1,1) diagonal,
# in the order PyGW enumerates them (kqmesh.py:219-224).
_TET0 = np.array(
    [
        [[0, 0, 0], [0, 0, 1], [0, 1, 1], [1, 1, 1]],
        [[0, 0, 0], [0, 1, 1], [0, 1, 0], [1, 1, 1]],
        [[0, 0, 0], [0, 1, 0], [1, 1, 0], [1, 1, 1]],
        [[0, 0, 0], [1, 1, 0], [1, 0, 0], [1, 1, 1]],
        [[0, 0, 0], [1, 0, 0], [1, 0, 1], [1, 1, 1]],
        [[0, 0, 0], [1, 0, 1], [0, 0, 1], [1, 1, 1]],
    ],
    dtype=np.int64,
)


def k2indx(k, div):
    """Linear index of integer mesh coordinates (for_kpts.f90:1-6)."""
    return (int(k[0]) * int(div[1]) + int(k[1])) * int(div[2]) + int(k[2])


def indx2k(indx, div):
    """Integer mesh coordinates of a linear index (for_kpts.f90:8-18)."""
    k2 = indx % div[2]
    i1 = indx // div[2]
    return np.array([i1 // div[1], i1 % div[1], k2], dtype=np.int64)


def shortest_diagonal(div, gbas=None):
    """Index of the shortest main diagonal of a mesh cell (kqmesh.py:203-214).

    ``gbas`` are the reciprocal lattice vectors as rows (identity = simple
    cubic, for which all four diagonals tie and the first one wins, as
    ``argmin`` does in the reference).
    """
    gbas = np.eye(3) if gbas is None else np.asarray(gbas, dtype=float)
    p0 = np.array([[0, 0, 0, 0, 1, 1, 1, 1], [0, 0, 1, 1, 0, 0, 1, 1], [0, 1, 0, 1, 0, 1, 0, 1]])
    diag = np.zeros(4)
    for i in range(4):
        sm = np.dot([(p0[k, i] - p0[k, 7 - i]) / float(div[k]) for k in range(3)], gbas)
        diag[i] = np.sum(sm ** 2)
    return int(np.argmin(diag))


def rotated_tetrahedra(mnd):
    """The unit-cube tetrahedra rotated onto diagonal ``mnd`` (kqmesh.py:226-240)."""
    tet = np.zeros_like(_TET0)
    if mnd == 0:
        tet[:] = _TET0
    elif mnd == 1:
        tet[:, :, 0] = _TET0[:, :, 0]
        tet[:, :, 1] = _TET0[:, :, 2]
        tet[:, :, 2] = 1 - _TET0[:, :, 1]
    elif mnd == 2:
        tet[:, :, 0] = _TET0[:, :, 0]
        tet[:, :, 1] = 1 - _TET0[:, :, 2]
        tet[:, :, 2] = _TET0[:, :, 1]
    elif mnd == 3:
        tet[:, :, 0] = _TET0[:, :, 0]
        tet[:, :, 1] = 1 - _TET0[:, :, 1]
        tet[:, :, 2] = 1 - _TET0[:, :, 2]
    else:
        raise ValueError("mnd must be 0..3")
    return tet


def build_tetc(div, gbas=None):
    """``tetc[4, 6*nkp]`` (Fortran order, int32, 0-based), kqmesh.py:242-257.

    Tetrahedron ``6*ik + t`` belongs to the cube whose origin is mesh point
    ``ik``; corner ``i`` is ``(orig + tet[t, i]) mod div``.
    """
    div = np.asarray(div, dtype=np.int64)
    tet = rotated_tetrahedra(shortest_diagonal(div, gbas))
    nkp = int(np.prod(div))
    tetc = np.zeros((4, 6 * nkp), dtype=np.int32, order="F")
    for ik, iii in enumerate(itertools.product(range(div[0]), range(div[1]), range(div[2]))):
        orig = np.array(iii, dtype=np.int64)
        for t in range(6):
            for i in range(4):
                corn = (orig + tet[t, i, :]) % div
                tetc[i, 6 * ik + t] = k2indx(corn, div)
    return tetc


def build_kqid(div):
    """``kqid[ik, iq]`` = index of k−q (for_kpts.f90:21-45), int32, Fortran order."""
    div = np.asarray(div, dtype=np.int64)
    nkp = int(np.prod(div))
    ks = np.array([indx2k(i, div) for i in range(nkp)])
    kmq = (ks[:, None, :] - ks[None, :, :]) % div  # [ik, iq, 3]
    kqid = (kmq[..., 0] * div[1] + kmq[..., 1]) * div[2] + kmq[..., 2]
    return np.asfortranarray(kqid.astype(np.int32))


def kpoint_coords(div):
    """Fractional coordinates j/n of every mesh point, shape [nkp, 3] (Γ-centred)."""
    div = np.asarray(div, dtype=np.int64)
    nkp = int(np.prod(div))
    return np.array([indx2k(i, div) / div for i in range(nkp)], dtype=float)


class KQmesh:
    """Minimal stand-in for PyGW's ``KQmesh`` with the attributes the
    polarization path reads: ``ndiv``, ``tetc``, ``kqid``, ``kii_ind``,
    ``ntet``."""

    def __init__(self, div, gbas=None):
        self.ndiv = np.asarray(div, dtype=np.int64)
        self.nkp = int(np.prod(self.ndiv))
        self.tetc = build_tetc(self.ndiv, gbas)
        self.kqid = build_kqid(self.ndiv)
        self.kii_ind = np.arange(self.nkp, dtype=np.int64)
        self.ntet = 6 * self.nkp
