"""Generate golden vectors for calc_selfc from the reference's own code.

Run where the reference's source tree is available:

    python tests/golden/make_calc_selfc_golden.py --reference <PyGW source tree>

As make_calc_eps_golden.py does for calc_eps, this reads the text of
``MatrixElements2Band.calc_selfc`` (pygw.py:3299-3412) and of
``Compute_selfc_inside`` (mcommon.py:80-165), rewrites their Python 2 print
statements, and runs them on seeded inputs with stand-in objects.  What the
reference computes in Python is then the reference's own arithmetic: the
mwm contraction with its q = 0 head and wing terms, the energies at k − q
(core states first), the spline interpolation of the iopfreq 4 branch and the
reshape/product of the SVD branch.  The three Fortran kernels it calls
(fnc.f90: all_fr_convolutions, few_fr_convolutions, many_fr_convolutions,
with fr_convolution2) cannot be compiled here; they run from their Fortran
text through ``f90py`` (beside this script), with the f2py calling
convention the reference uses (outputs returned, sizes from the shapes), so
the golden values are the reference's own statements end to end.

Cases: a finite q; q = 0 with head and wings on a dense frequency mesh
(iopfreq 4, the spline branch); a finite q in an SVD basis; and a finite q on
the dense mesh with W Hermitian at each frequency (mwm real up to rounding,
so the spline of its imaginary part is skipped) and no core states (no core
block from calc_minm).  Output: ``calc_selfc_golden.npz`` beside this script.
"""
import io
import itertools
import math
import os
import sys
import timeit
import warnings

import numpy as np
import scipy.interpolate
import scipy.linalg

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import f90py  # noqa: E402
f90py.POISON = True     # a read of storage never written shows as NaN, or raises
import refsrc  # noqa: E402
from refsrc import NS  # noqa: E402

PYGW = refsrc.reference_file("pygw.py")
MCOMMON = refsrc.reference_file("mcommon.py")
OUT = os.path.join(HERE, "calc_selfc_golden.npz")


def _fnc(enks):
    """The reference's Fortran kernels (fnc.f90), run from their source text,
    behind the f2py calling convention; each records the energies the
    reference handed it (once per k-point)."""
    procs, _ = f90py.load([refsrc.reference_file("fnc.f90")],
                          ["all_fr_convolutions", "few_fr_convolutions", "many_fr_convolutions"], math.atan, math.log)
    FA = f90py.FArr

    def seen(enk):
        if not enks or not np.array_equal(enks[-1], enk):
            enks.append(np.array(enk))

    def farr(a, dtype):
        a = np.asfortranarray(np.asarray(a, dtype=dtype))
        return FA(a, (1,) * a.ndim)

    def i4(x):
        return np.array(x, dtype=np.int32)

    def all_fr_convolutions(enk, mwm, omega, womeg):
        seen(enk)
        nom, nb1, nb2 = np.shape(mwm)
        sc = FA(np.zeros((nb1, nom), dtype=np.complex128, order="F"), (1, 1))
        procs["all_fr_convolutions"](sc, farr(enk, np.float64), farr(mwm, np.complex128), farr(omega, np.float64),
                                     farr(womeg, np.float64), i4(nb1), i4(nb2), i4(nom))
        return sc.a

    def few_fr_convolutions(enk, mwmp, mwm_iom, omega, omega_iom, womeg):
        seen(enk)
        nb2, nom = np.shape(mwmp)
        res = np.zeros((), dtype=np.complex128)
        procs["few_fr_convolutions"](res, farr(enk, np.float64), farr(mwmp, np.complex128),
                                     farr(mwm_iom, np.complex128), farr(omega, np.float64),
                                     np.array(float(omega_iom)), farr(womeg, np.float64), i4(nom), i4(nb2))
        return res[()]

    def many_fr_convolutions(enk, Ul, omega, womeg):
        seen(enk)
        nl, nom = np.shape(Ul)
        nb2 = len(enk)
        sc = FA(np.zeros((nl, nb2, nom), dtype=np.complex128, order="F"), (1, 1, 1))
        procs["many_fr_convolutions"](sc, farr(enk, np.float64), farr(Ul, np.complex128), farr(omega, np.float64),
                                      farr(womeg, np.float64), i4(nom), i4(nl), i4(nb2))
        return sc.a
    return NS(all_fr_convolutions=all_fr_convolutions, few_fr_convolutions=few_fr_convolutions,
              many_fr_convolutions=many_fr_convolutions)


def load(saved, enks):
    ns = {}
    exec("from numpy import *", ns)
    ns.update(interpolate=scipy.interpolate, linalg=scipy.linalg, la=np.linalg, timer=timeit.default_timer,
              itertools=itertools, sys=sys, FORT=True, fnc=_fnc(enks),
              save=lambda path, a: saved.append(np.array(a)))
    ns["mcmn"] = NS(Compute_selfc_inside=refsrc.load(MCOMMON, "def Compute_selfc_inside(", "", ns, "Compute_selfc_inside"))
    return refsrc.load(PYGW, "    def calc_selfc(self,", "    ", ns, "calc_selfc")


def case(rng, iq, npb=16, nkp=4, ibgw=1, nbgw=3, ncg_c=1, nbands_c=6, nom=5, nl=None, dense=False,
         hermitian=False):
    nb1, nb2 = nbgw - ibgw, nbands_c
    nw = nom if nl is None else nl
    W = 0.3 * (rng.standard_normal((npb, npb, nw)) + 1j * rng.standard_normal((npb, npb, nw)))
    if hermitian:            # W Hermitian at each frequency: mwm real up to rounding
        W = 0.5 * (W + np.conj(W.transpose(1, 0, 2)))
    M = 0.2 * (rng.standard_normal((nkp, nb1, nb2, npb)) + 1j * rng.standard_normal((nkp, nb1, nb2, npb)))
    Ebnd = np.sort(rng.uniform(-1.0, 2.0, (1, nkp, nbands_c)), axis=2)
    core_e = [-8.0 - rng.uniform(0, 1)]
    kqid = np.stack([np.arange(nkp), rng.permutation(nkp)], axis=1)          # k − q index per q
    omega = np.geomspace(0.02, 20.0, nom)
    womeg = np.gradient(omega)
    omega_p = np.geomspace(0.01, 40.0, 40) if dense else omega
    womeg_p = np.gradient(omega_p)
    Ul = rng.standard_normal((nl, nom)) / np.sqrt(nom) if nl is not None else None
    head = epsw1 = epsw2 = None
    if iq == 0:
        head = rng.standard_normal(nw) + 1j * rng.standard_normal(nw)
        epsw1 = 0.3 * (rng.standard_normal((npb, nw)) + 1j * rng.standard_normal((npb, nw)))
        epsw2 = 0.3 * (rng.standard_normal((npb, nw)) + 1j * rng.standard_normal((npb, nw)))
    singc1, singc2, Vol = 0.7, 1.3, 250.0

    def calc_minm(ik, iq_, band_limits, kind, *a):
        # valence, core (None without core states, as calc_minm returns it)
        return M[ik][:, ncg_c:, :].copy(), (M[ik][:, :ncg_c, :].copy() if ncg_c else None)

    me = NS(singc1=singc1, singc2=singc2, calc_minm=calc_minm)
    kqm = NS(qlistc=np.zeros((2, 3), dtype=int), LCMq=1, qlist=np.zeros((3, 3)), weight=np.ones(nkp),
             kirlist=np.zeros((nkp, 3), dtype=int), LCM=1, k_ind=np.arange(nkp), kqid=kqid, kii_ind=np.arange(nkp))
    ks = NS(ibgw=ibgw, nbgw=nbgw, nbands_c=nbands_c, ncg_c=ncg_c, Ebnd=Ebnd)
    core = NS(corind=np.array([[0, 0, 0]]), eig_core=[[core_e]])
    fr = NS(omega=omega, womeg=womeg, iopfreq=4 if dense else 1, omega_precise=omega_p, womeg_precise=womeg_p)
    saved, enks = [], []
    sc_p = load(saved, enks)(me, iq, W, epsw1, epsw2, None if head is None else head.copy(), NS(nat=1), None,
                       NS(Vol=Vol), kqm, ks, None, NS(inverse_indgq=lambda q: None), NS(big_l=[[0]]), core, None,
                       fr, "", None, Ul, io.StringIO())
    enk = np.array(enks)
    assert enk.shape == (nkp, nb2)
    out = dict(W=W, M=M, Ebnd=Ebnd, core_e=np.array(core_e), kqid=kqid, omega=omega, womeg=womeg,
               mwm=np.array(saved), sc_p=np.asarray(sc_p), enk=enk,
               wkq=np.array(1.0 / 3), coefs=np.array([singc1 * np.sqrt(4 * np.pi / Vol), singc2 * 4 * np.pi / Vol]))
    if iq == 0:
        out.update(head=head, epsw1=epsw1, epsw2=epsw2)
    if dense:
        out.update(omega_p=omega_p, womeg_p=womeg_p)
    if Ul is not None:
        out.update(Ul=Ul)
    return out


def main():
    warnings.filterwarnings("ignore", category=SyntaxWarning)    # escape sequences in the reference's docstrings
    rng = np.random.default_rng(20261204)
    cases = {
        "q": case(rng, 1),
        "q0dense": case(rng, 0, dense=True),
        "svd": case(rng, 1, nl=3),
        "densereal": case(rng, 1, ncg_c=0, dense=True, hermitian=True),
    }
    flat = {f"{c}.{k}": v for c, d in cases.items() for k, v in d.items()}
    np.savez_compressed(OUT, **flat)
    print(f"wrote {OUT}: " + ", ".join(f"{k}{tuple(np.shape(v))}" for k, v in flat.items()))


if __name__ == "__main__":
    refsrc.run(main)
