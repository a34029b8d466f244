"""Generate golden vectors for the SVD frequency basis from the reference's own code.

Run where the reference's source tree is available:

    python tests/golden/make_svd_golden.py --reference <PyGW source tree>

Runs the text of ``svd_functions`` (pygw.py:3478-3501) and of
``Give2TanMesh`` (mcommon.py:13-31) on three Matsubara meshes, the third with a
lower frequency bound that Give2TanMesh clamps.  Two Python 2
forms are rewritten: print statements become print() calls, and the integer
division ``len(iom)/2`` becomes ``len(iom)//2`` (what it computes under
Python 2).  The reference's ``linalg`` there is scipy.linalg.  Output:
``svd_golden.npz`` beside this script.
"""
import io
import os
import sys
import warnings

import numpy as np
import scipy.linalg
import scipy.optimize

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refsrc  # noqa: E402
from refsrc import NS  # noqa: E402

PYGW = refsrc.reference_file("pygw.py")
MCOMMON = refsrc.reference_file("mcommon.py")
OUT = os.path.join(HERE, "svd_golden.npz")


def load():
    ns = {}
    exec("from numpy import *", ns)
    ns.update(optimize=scipy.optimize, linalg=scipy.linalg)
    give2tan = refsrc.load(MCOMMON, "def Give2TanMesh(", "", ns, "Give2TanMesh")
    ns["mcmn"] = NS(Give2TanMesh=give2tan)
    return give2tan, refsrc.load(PYGW, "def svd_functions(", "", ns, "svd_functions", replace=[("len(iom)/2", "len(iom)//2")])


def main():
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    give2tan, svd_functions = load()
    out = {}
    for name, (nom, om_min, om_max, om_nom, cut) in {
            "a": (32, 1e-3, 20.0, 60, 1e-10),
            "b": (48, 5e-4, 40.0, 80, 1e-8),
            # om_min above L * Nw * tan(pi / 2Nw)^2 / 4: Give2TanMesh clamps it
            "c": (24, 0.1, 1.0, 10, 1e-8)}.items():
        x = np.polynomial.legendre.leggauss(nom)
        t = 0.5 * (x[0] + 1.0)
        iomega = 0.02 * t / (1.0 - t + 1e-3)                   # a Matsubara-like mesh, dense near 0
        wiomeg = 0.02 * 0.5 * x[1] * (1.0 + 1e-3) / (1.0 - t + 1e-3) ** 2
        om, dom = give2tan(om_min, om_max, om_nom)
        Ul, dUl = svd_functions(iomega, wiomeg, om_min, om_max, om_nom, cut, io.StringIO())
        out.update({f"{name}.iomega": iomega, f"{name}.wiomeg": wiomeg,
                    f"{name}.args": np.array([om_min, om_max, om_nom, cut]),
                    f"{name}.om": om, f"{name}.dom": dom, f"{name}.Ul": Ul, f"{name}.dUl": dUl})
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: " + ", ".join(f"{k}{tuple(np.shape(v))}" for k, v in out.items()))


if __name__ == "__main__":
    refsrc.run(main)
