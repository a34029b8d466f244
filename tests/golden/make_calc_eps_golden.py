"""Generate golden vectors for calc_eps from the reference's own code.

Run where the reference's source tree is available:

    python tests/golden/make_calc_eps_golden.py --reference <PyGW source tree>

The reference's driver is Python 2 with f2py modules, so it cannot be
imported here.  This script reads the text of
``MatrixElements2Band.calc_eps`` (pygw.py:3039-3297) at run time, rewrites
its Python 2 print statements as print() calls (nothing else is changed),
and runs the method with numpy/scipy in place of the reference's star
imports and with small stand-in objects for the parts of the reference that
are not on this path (the product basis, the mesh and band objects, and
``calc_minm``, which returns seeded random matrix elements).  The weights
``kcw`` are seeded random numbers too: the contraction does not depend on
where they come from.  The inputs and the reference's outputs are written to
``calc_eps_golden.npz`` beside this script; nothing of the reference's source
is stored.

Cases: a finite q, q = 0 (head and wings from seeded momentum matrix
elements), q = 0 in an SVD frequency basis (Ul, dUl), and q = 0 with two
core states (calc_minm's core block ``minc0`` ahead of the valence one, core
levels from ``core.eig_core``, core-to-empty momentum elements ``mmatcv``)
and momentum elements stored from band ``mst`` = 1 on.
"""
import io
import itertools
import os
import sys
import timeit

import numpy as np
import scipy.linalg

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import refsrc  # noqa: E402
from refsrc import NS, load, reference_file  # noqa: E402

REF = reference_file("pygw.py")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "calc_eps_golden.npz")


def load_calc_eps():
    ns = {}
    exec("from numpy import *", ns)
    ns.update(linalg=scipy.linalg, la=np.linalg, timer=timeit.default_timer, itertools=itertools, sys=sys,
              Save_eps=False, ForceReal=False, save=np.save)
    return load(REF, "    def calc_eps(self,", "    ", ns, "calc_eps")


def case(rng, iq, nkp, nvbm, ncbm, nb2, npb, nom, nl=None, ncg=0, mst=0):
    """Inputs in the reference's layouts and the reference's calc_eps result."""
    nbmaxpol = ncbm + nb2
    nb1 = ncg + nvbm                               # core states first
    nw = nom if nl is None else nl                 # kcw's last axis: frequencies or basis functions
    M = 0.08 * (rng.standard_normal((nkp, nvbm, nb2, npb)) + 1j * rng.standard_normal((nkp, nvbm, nb2, npb)))
    Mc = None
    if ncg:                                        # core-to-empty matrix elements (calc_minm's minc0)
        Mc = 0.05 * (rng.standard_normal((nkp, ncg, nb2, npb)) + 1j * rng.standard_normal((nkp, ncg, nb2, npb)))
    kcw = np.asfortranarray(rng.uniform(0.0, 1.0, (nb1, nb2, nkp, nw)))
    Ebnd = np.sort(rng.uniform(-1.0, 2.0, (1, nkp, nbmaxpol)), axis=2)
    Ebnd[0, :, :nvbm] -= 1.0                       # occupied below the empty bands
    Vol = 250.0
    omega = np.geomspace(0.01, 10.0, nom)
    Ul = dUl = None
    if nl is not None:
        Ul = rng.standard_normal((nl, nom)) / np.sqrt(nom)
        dUl = np.linalg.pinv(Ul)                   # (nom, nl)
    head_in = mmatvv = mmatcv = pm = None
    ecore = np.linspace(-4.0, -3.0, ncg)           # core levels, eig_core[0][0][ic]
    corind = np.array([[0, 0, ic] for ic in range(ncg)], dtype=int).reshape(ncg, 3)
    if iq == 0:
        head_in = (rng.uniform(0.5, 2.0, nw) + 0.1j * rng.standard_normal(nw)).astype(complex)
        # momentum matrix elements stored from band mst on
        shp = (nkp, nbmaxpol - mst, nvbm, 3)
        mmatvv = 0.3 * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp))
        shp = (nkp, nbmaxpol - mst, ncg, 3)
        mmatcv = 0.3 * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) if ncg else np.zeros(shp, complex)
        # pm as pygw.py:3089-3093 and 3120-3141 form it (restated to hand the
        # same vector to the oracle)
        coefw = 2.0 * np.sqrt(np.pi / Vol)
        pm = np.zeros((nkp, nb1 * nb2), dtype=complex)
        for ik in range(nkp):
            enk = np.concatenate([ecore, Ebnd[0, ik, :nbmaxpol]])
            mmc = np.sum(mmatcv[ik, ncbm - mst:nbmaxpol - mst, :, :], axis=2) * (coefw / np.sqrt(3.0))
            mmv = np.sum(mmatvv[ik, ncbm - mst:nbmaxpol - mst, :, :], axis=2) * (coefw / np.sqrt(3.0))
            ie12 = 0
            for ie1 in range(ncg + nvbm):
                for ie2 in range(ncbm, nbmaxpol):
                    edif = enk[ie1] - enk[ie2 + ncg]
                    if abs(edif) > 1e-10:
                        pm[ik, ie12] = (mmc[ie2 - ncbm, ie1] if ie1 < ncg else mmv[ie2 - ncbm, ie1 - ncg]) / edif
                    ie12 += 1

    me = NS(barcvm=np.zeros((1, npb)),
            calc_minm=lambda ik, *a: (M[ik].copy(), None if Mc is None else Mc[ik].copy()))
    strc = NS(nat=1)
    pb = NS(big_l=[[0, 1]])
    pw = NS(inverse_indgq=lambda q: None)
    kqm = NS(qlistc=np.zeros((2, 3), dtype=int), LCMq=1, kii_ind=np.arange(nkp), kqid=np.zeros((nkp, 2), dtype=int))
    ks = NS(nomax_numin=(nvbm - 1, ncbm), ncg_p=ncg, nbmaxpol=nbmaxpol, Ebnd=Ebnd)
    core = NS(corind=corind, eig_core=[[list(ecore)]])
    latgen = NS(Vol=Vol)
    fr = NS(omega=omega)
    hq = None
    if iq == 0:
        hq = (head_in.copy(), mmatcv, mmatvv, mst)
    fout = io.StringIO()
    eps, epsw1, epsw2, head = load_calc_eps()(me, iq, hq, strc, None, latgen, kqm, ks, None, pw, pb, core, None, fr,
                                                kcw, "", dUl, Ul, fout)
    out = dict(M=M if Mc is None else np.concatenate([Mc, M], axis=1), kcw=kcw, eps=np.asarray(eps))
    if iq == 0:
        out.update(pm=pm, head_in=head_in, epsw1=epsw1, epsw2=epsw2, head=np.asarray(head),
                   Ebnd=Ebnd, mmatvv=mmatvv, mmatcv=mmatcv, mst=mst, ecore=ecore, Vol=Vol,
                   nomax_numin=np.array([nvbm - 1, ncbm]))
    if nl is not None:
        out.update(Ul=Ul, dUl=dUl)
    return out


def main():
    rng = np.random.default_rng(20261203)
    cases = {
        "q": case(rng, 1, nkp=6, nvbm=3, ncbm=3, nb2=5, npb=24, nom=4),
        "q0": case(rng, 0, nkp=6, nvbm=3, ncbm=3, nb2=5, npb=24, nom=4),
        "q0svd": case(rng, 0, nkp=6, nvbm=3, ncbm=3, nb2=5, npb=24, nom=6, nl=4),
        "q0core": case(rng, 0, nkp=6, nvbm=3, ncbm=3, nb2=5, npb=24, nom=4, ncg=2, mst=1),
    }
    flat = {f"{c}.{k}": np.asarray(v) for c, d in cases.items() for k, v in d.items()}
    np.savez_compressed(OUT, **flat)
    print(f"wrote {OUT}: " + ", ".join(f"{k}{tuple(v.shape)}" for k, v in flat.items()))


if __name__ == "__main__":
    refsrc.run(main)
