"""Generate golden vectors for the host side of Polarization_weights from the
reference's own code.

Run where the reference's source tree is available:

    python tests/golden/make_polarization_weights_golden.py --reference <PyGW source tree>

Runs the text of ``Polarization_weights`` (pygw.py:3416-3476) with print
statements rewritten, on seeded band energies with core states and a
symmetry-reduced k-point map.  The Fortran weight routines it calls
(``ft.bz_calcqdepw_par2`` / ``par3``) are replaced by recorders: the golden
values are the arguments the reference hands them — above all the energy
array ``enk[nbnd, nkp]`` assembled from core and band energies — which the
product's host code must reproduce.  Output: ``polarization_weights_golden.npz``.
"""
import io
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refsrc  # noqa: E402
from refsrc import NS, load, reference_file  # noqa: E402

PYGW = reference_file("pygw.py")
OUT = os.path.join(HERE, "polarization_weights_golden.npz")


def main():
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    calls = []

    def par2(*a):
        calls.append(("par2", a))
        return np.zeros(1)

    def par3(*a):
        calls.append(("par3", a))
        return np.zeros(1)

    ns = {}
    exec("from numpy import *", ns)
    ns.update(ft=NS(bz_calcqdepw_par2=par2, bz_calcqdepw_par3=par3), sys=NS(exit=lambda *a: None))
    pw = load(PYGW, "def Polarization_weights(", "", ns, "Polarization_weights")

    rng = np.random.default_rng(20261205)
    nkp, nirkp, ncg_p, nbmaxpol = 8, 5, 2, 7
    kii_ind = np.array([0, 1, 1, 2, 3, 3, 4, 0])                      # k-point → irreducible point
    Ebnd = np.sort(rng.uniform(-1.0, 2.0, (1, nirkp, 10)), axis=2)
    eig_core = [[[-20.0, -15.0], [-30.0]]]                            # [isp][atom][core state]
    corind = np.array([[1, 0, 0], [0, 0, 1]])                         # (atom, -, state) per core state
    ks = NS(nomax_numin=(3, 2), ncg_p=ncg_p, nbmaxpol=nbmaxpol, Ebnd=Ebnd, EF=0.1)
    kqm = NS(kii_ind=kii_ind, kqid=np.stack([np.arange(nkp), rng.permutation(nkp)], axis=1),
             tetc=rng.integers(0, nkp, (4, 6 * nkp)))
    core = NS(corind=corind, eig_core=eig_core)
    fr = NS(omega=np.geomspace(0.01, 10.0, 5))
    dUl = rng.standard_normal((5, 3))
    pw(1, ks, kqm, core, fr, 0, 1, None, io.StringIO())
    pw(0, ks, kqm, core, fr, 0, 1, dUl, io.StringIO())
    (k2, a2), (k3, a3) = calls
    assert (k2, k3) == ("par2", "par3")
    np.savez_compressed(OUT, Ebnd=Ebnd, kii_ind=kii_ind, corind=corind, eig_core0=np.array(eig_core[0][0]),
                        eig_core1=np.array(eig_core[0][1]), nomax_numin=np.array(ks.nomax_numin), ncg_p=ncg_p,
                        nbmaxpol=nbmaxpol, kqid=kqm.kqid, enk=np.asarray(a2[0]), kqid_par2=np.asarray(a2[2]),
                        args_par2=np.array([a2[1], a2[3], a2[4], a2[5]]), enk_par3=np.asarray(a3[0]),
                        kqid_par3=np.asarray(a3[2]))
    print(f"wrote {OUT}: enk{np.shape(a2[0])}")


if __name__ == "__main__":
    refsrc.run(main)
