"""Generate golden vectors for the tetrahedra and the k − q table from the
reference's own code.

Run where the reference's source tree is available:

    python tests/golden/make_mesh_golden.py --reference <PyGW source tree>

Runs the text of ``KQmesh.tetra`` (kqmesh.py:188-380) on several meshes and
reciprocal bases, with its Python branch for the k − q table (``FORT``
false).  Python 2 forms rewritten: print statements become print() calls and
``d.has_key(x)`` becomes ``x in d``.  The stand-in object supplies the mesh
attributes ``tetra`` reads (no symmetry: every k-point is its own
irreducible point) and ``k2indx`` / ``indx2k`` as kqmesh.py:17-24 define
them, with ``//`` for their Python 2 integer divisions; ``fkp.k2indx``
(for_kpts.f90:2-7) is the same formula.  Output: ``mesh_golden.npz`` beside
this script (tetc, kqid and the chosen diagonal per case).
"""
import io
import itertools
import os
import sys
import timeit
import warnings
from functools import reduce

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
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


def load():
    ns = {}
    exec("from numpy import *", ns)
    ns.update(itertools=itertools, timer=timeit.default_timer, FORT=False, reduce=reduce, lcm=np.lcm,
              fkp=NS(k2indx=lambda k, div: (k[0] * div[1] + k[1]) * div[2] + k[2]))
    return refsrc.load(KQMESH, "    def tetra(self,", "    ", ns, "tetra")


def main():
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    tetra = load()
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
        tetra(m, NS(ortho=False), NS(lattice="P  "), io.StringIO())
        out.update({f"{name}.div": np.array(div), f"{name}.gbas": np.array(gbas, dtype=float),
                    f"{name}.tetc": np.asarray(m.tetc), f"{name}.kqid": np.asarray(m.kqid),
                    f"{name}.mnd": np.array(m.mnd)})
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: " + ", ".join(f"{k}={int(v)}" for k, v in out.items() if k.endswith(".mnd")))


if __name__ == "__main__":
    main()
