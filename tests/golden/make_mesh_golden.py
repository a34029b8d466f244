"""Generate golden vectors for the tetrahedra and the k − q table from the
reference's own code.

Run where the reference's source tree is available:

    python tests/golden/make_mesh_golden.py --reference <PyGW source tree>

Runs the text of ``KQmesh.tetra`` (kqmesh.py:188-380) on several meshes and
reciprocal bases, once with its Python branch for the k − q table (``FORT``
false) and once with its Fortran branch, and requires the two to agree.
Python 2 forms rewritten: print statements become print() calls and
``d.has_key(x)`` becomes ``x in d``.  The stand-in object supplies the mesh
attributes ``tetra`` reads (no symmetry: every k-point is its own
irreducible point) and ``k2indx`` / ``indx2k`` as kqmesh.py:17-24 define
them, with ``//`` for their Python 2 integer divisions.  The Fortran it calls
(``fkp.k2indx`` and ``fkp.k_m_q_id``, for_kpts.f90:2-45; no compiler here)
runs from its source text through ``f90py`` beside this script, behind the
f2py calling convention.  Output: ``mesh_golden.npz`` beside this script
(tetc, kqid and the chosen diagonal per case).
"""
import io
import itertools
import math
import os
import sys
import timeit
import warnings
from functools import reduce

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import f90py  # noqa: E402
f90py.POISON = True     # a read of storage never written shows as NaN, or raises
import refsrc  # noqa: E402
from refsrc import NS  # noqa: E402

KQMESH = refsrc.reference_file("kqmesh.py")
OUT = os.path.join(HERE, "mesh_golden.npz")


class Mesh:
    """The attributes of a KQmesh that ``tetra`` reads, for a mesh without symmetry."""

    def __init__(self, div, gbas):
        self.ndiv = np.array(div, dtype=int)
        self.shift = np.zeros(4, dtype=int)
        self.gbas = np.array(gbas, dtype=float)
        nkp = int(np.prod(div))
        self.kii_ind = np.arange(nkp)
        self.k_ind = np.arange(nkp)
        self.weight = np.ones(nkp)
        self.sym = [np.eye(3)]
        self.LCM = int(np.lcm.reduce(self.ndiv))
        self.k2cartes = np.eye(3)

    def k2indx(self, k):
        return (k[0] * self.ndiv[1] + k[1]) * self.ndiv[2] + k[2]

    def indx2k(self, ind):
        k2 = ind % self.ndiv[2]
        i1 = ind // self.ndiv[2]
        k1 = i1 % self.ndiv[1]
        k0 = i1 // self.ndiv[1]
        return np.array([k0, k1, k2])


def _fkp():
    """The reference's for_kpts.f90 routines, run from their source text."""
    procs, _ = f90py.load([refsrc.reference_file("for_kpts.f90")], ["k2indx", "k_m_q_id"], math.atan, math.log)

    def ivec(a):
        return f90py.FArr(np.asarray(a, dtype=np.int32).copy(), (1,))

    def k2indx(k, div):
        out = np.zeros((), dtype=np.int32)
        procs["k2indx"](out, ivec(k), ivec(div))
        return int(out)

    def k_m_q_id(div, nkp):
        kqid = f90py.FArr(np.zeros((nkp, nkp), dtype=np.int32, order="F"), (1, 1))
        procs["k_m_q_id"](kqid, ivec(div), np.array(nkp, dtype=np.int32))
        return kqid.a
    return NS(k2indx=k2indx, k_m_q_id=k_m_q_id)


def load():
    ns = {}
    exec("from numpy import *", ns)
    ns.update(itertools=itertools, timer=timeit.default_timer, FORT=False, reduce=reduce, lcm=np.lcm, fkp=_fkp())
    return refsrc.load(KQMESH, "    def tetra(self,", "    ", ns, "tetra"), ns


def main():
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    tetra, ns = load()
    cases = {
        "cubic444": ((4, 4, 4), np.eye(3)),
        "mixed345": ((3, 4, 5), np.eye(3)),
        # skewed reciprocal bases: each of the other three cube diagonals the shortest
        "skew1": ((3, 3, 3), [[1, 0, 0], [0, 1, 0.5], [0.5, 0, 1]]),
        "skew2": ((3, 3, 3), [[1, 0.5, 0], [0, 1, 0.5], [0, 0, 1]]),
        "skew3": ((3, 3, 3), [[1, 0, 0], [0, 1, 0], [0.5, -0.5, 1]]),
        "skew2b": ((4, 3, 2), [[1, 0, -0.5], [0, 1, 0.5], [0, 0, 1]]),
    }
    out = {}
    for name, (div, gbas) in cases.items():
        m = Mesh(div, gbas)
        ns["FORT"] = True                 # k − q table from the Fortran branch
        tetra(m, NS(ortho=False), NS(lattice="P  "), io.StringIO())
        kqid_fortran = np.asarray(m.kqid).copy()
        m = Mesh(div, gbas)
        ns["FORT"] = False                # … and from the Python branch
        tetra(m, NS(ortho=False), NS(lattice="P  "), io.StringIO())
        assert np.array_equal(np.asarray(m.kqid), kqid_fortran), name
        out.update({f"{name}.div": np.array(div), f"{name}.gbas": np.array(gbas, dtype=float),
                    f"{name}.tetc": np.asarray(m.tetc), f"{name}.kqid": np.asarray(m.kqid),
                    f"{name}.mnd": np.array(m.mnd)})
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: " + ", ".join(f"{k}={int(v)}" for k, v in out.items() if k.endswith(".mnd")))


if __name__ == "__main__":
    refsrc.run(main)
