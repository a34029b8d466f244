"""Generate golden tetrahedron weights from the reference's own Fortran statements.

Run where the reference's source tree is available:

    python tests/golden/make_weights_golden.py --reference <PyGW source tree>

Neither this container nor the GPU machine has a Fortran compiler, so the
reference's ``bz_calcqdepw_par2`` (for_tetrahedra.f90:390-464) and everything
it calls (``convw1t_par``, ``surfnodes`` … ``sortnodes``, ``generictetra_par``,
``stweight_imag_par``, ``stweight_itaylor_par``, ``sorteq``: for_tetrahedra2.f90
and for_tetrahedra3.f90) are read from the reference's files and executed
statement by statement through ``f90py`` (beside this script), which keeps
every variable's declared kind and passes arguments by reference with the
storage association compiled Fortran uses.  The only substitution is the
arc tangent and logarithm: each case is run twice, once with the C library's
``atan``/``log`` (what a compiled reference calls) and once with the portable
implementations the oracle and the GPU kernels share, so that the oracle's
restatement can be compared bit for bit with the reference's statements.

The same is done for ``bz_calcqdepw_par3`` (for_tetrahedra.f90:466-542), the
weights projected on an SVD frequency basis ``dUl`` (seeded, three
functions), with ``matmul`` summed over the frequencies in ascending order.

Cases (seeded synthetic band structures with the workload generator's
shapes): C1-like bands on a 2³ k-mesh, a stress case whose partially
occupied bands give polyhedra with 4, 6 and 8 nodes, and a degenerate case
(energies on a grid of 0.25: values at EF, equal corners) with 5- and 7-node
polyhedra too; four imaginary frequencies each; a case with a core state
and an offset empty-band window (ncg = 1, numin = 1), three frequencies; and
a static-limit case at q = Γ (frequencies 0 and 1e-7, a band pair 1e-7
apart, a six-node polyhedron with two quadrilateral faces) that reaches the
branches the other cases leave unexecuted.  The statements run with
``f90py.POISON`` on, so a weight that depended on storage never written
would come out NaN (the script then stops).

Output: ``weights_golden.npz`` (inputs and the reference's ``kcw`` of par2
and par3 for each math variant); nothing of the reference's source is
stored.  ``--check-c1`` instead compares the oracle (with the reference's
layout of 7- and 8-node halves) with the reference's statements on the full
C1 problem and stores nothing; ``--coverage`` lists the statements of the
translated routines that no case executes and stores nothing.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
import f90py  # noqa: E402
f90py.POISON = True     # a read of storage never written shows as NaN, or raises
import refsrc  # noqa: E402
from refsrc import reference_file  # noqa: E402

OUT = os.path.join(HERE, "weights_golden.npz")
FILES = ["for_tetrahedra.f90", "for_tetrahedra2.f90", "for_tetrahedra3.f90"]


def reference_par2(math_impl):
    atan, log = math_impl
    procs, _ = f90py.load([reference_file(f) for f in FILES], ["bz_calcqdepw_par2"], atan, log)
    fn = procs["bz_calcqdepw_par2"]

    def run(enk, ef, kqid, ncg, nomx, numin, omega, tetc):
        enk = np.asfortranarray(enk, dtype=np.float64)
        tetc = np.asfortranarray(tetc, dtype=np.int32)
        nbnd, nkp = enk.shape
        ntet = tetc.shape[1]
        nom = len(omega)
        nb1, nb2 = ncg + nomx + 1, nbnd - ncg - numin
        kcw = f90py.FArr(np.zeros((nb1, nb2, nkp, nom), order="F"), (1, 1, 1, 1))
        i4 = lambda x: np.array(x, dtype=np.int32)     # noqa: E731
        fn(kcw, f90py.FArr(enk, (1, 1)), np.array(float(ef)), f90py.FArr(np.asarray(kqid, dtype=np.int32).copy(), (1,)),
           i4(ncg), i4(nomx), i4(numin), f90py.FArr(np.asarray(omega, dtype=np.float64).copy(), (1,)),
           f90py.FArr(tetc, (1, 1)), i4(nkp), i4(nom), i4(nbnd), i4(ntet))
        assert np.isfinite(kcw.a).all(), "the statements read storage they never wrote"
        return kcw.a.copy()
    return run


def reference_par3(math_impl):
    atan, log = math_impl
    procs, _ = f90py.load([reference_file(f) for f in FILES], ["bz_calcqdepw_par3"], atan, log)
    fn = procs["bz_calcqdepw_par3"]

    def run(enk, ef, kqid, ncg, nomx, numin, dUl, omega, tetc):
        enk = np.asfortranarray(enk, dtype=np.float64)
        tetc = np.asfortranarray(tetc, dtype=np.int32)
        nbnd, nkp = enk.shape
        ntet = tetc.shape[1]
        nom, nl = dUl.shape
        nb1, nb2 = ncg + nomx + 1, nbnd - ncg - numin
        kcw = f90py.FArr(np.zeros((nb1, nb2, nkp, nl), order="F"), (1, 1, 1, 1))
        i4 = lambda x: np.array(x, dtype=np.int32)     # noqa: E731
        fn(kcw, f90py.FArr(enk, (1, 1)), np.array(float(ef)), f90py.FArr(np.asarray(kqid, dtype=np.int32).copy(), (1,)),
           i4(ncg), i4(nomx), i4(numin), f90py.FArr(np.asfortranarray(dUl, dtype=np.float64), (1, 1)),
           f90py.FArr(np.asarray(omega, dtype=np.float64).copy(), (1,)), f90py.FArr(tetc, (1, 1)), i4(nkp), i4(nom),
           i4(nbnd), i4(ntet), i4(nl))
        assert np.isfinite(kcw.a).all(), "the statements read storage they never wrote"
        return kcw.a.copy()
    return run


def cases():
    from pygw_gb300 import synthetic as syn
    out = {}
    # C1-like bands, 2³ k-mesh, the last q point
    w = syn.scaled(syn.WORKLOADS["C1"], div=2, nbands=16, nocc=4, nom=4)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[-1]
    out["c1"] = dict(enk=b.enk(), ef=b.EF, kqid=p.kqm.kqid[:, iq], ncg=0, nomx=nomx, numin=numin,
                     omega=p.fr.omega, tetc=p.kqm.tetc)
    # stress: bands crossing the Fermi level everywhere on the same mesh, so
    # that the polyhedra {e <= EF <= f} take every node count
    rng = np.random.default_rng(11)
    nkp = p.kqm.nkp
    occ = rng.uniform(-0.6, 0.4, (3, nkp))
    emp = rng.uniform(-0.3, 0.9, (5, nkp))
    enk = np.concatenate([np.sort(occ, axis=0), np.sort(emp, axis=0)])
    out["stress"] = dict(enk=np.asfortranarray(enk), ef=0.0, kqid=p.kqm.kqid[:, iq], ncg=0, nomx=2, numin=0,
                         omega=np.array([0.02, 0.2, 2.0, 20.0]), tetc=p.kqm.tetc)
    # degenerate: the same bands on a grid of 0.25 (energies at EF and equal
    # corner values), whose polyhedra include 5- and 7-node ones
    rng = np.random.default_rng(156)
    occ = np.round(rng.uniform(-0.6, 0.4, (3, nkp)) * 4) / 4
    emp = np.round(rng.uniform(-0.3, 0.9, (5, nkp)) * 4) / 4
    enk = np.concatenate([np.sort(occ, axis=0), np.sort(emp, axis=0)])
    out["degenerate"] = dict(enk=np.asfortranarray(enk), ef=0.0, kqid=p.kqm.kqid[:, iq], ncg=0, nomx=2, numin=0,
                             omega=np.array([0.02, 0.2, 2.0, 20.0]), tetc=p.kqm.tetc)
    # band-window offsets: one core state below the bands (ncg = 1) and the
    # lowest band left out of the empty window (numin = 1)
    rng = np.random.default_rng(21)
    core = np.full((1, nkp), -5.0)
    occ = rng.uniform(-0.6, 0.4, (3, nkp))
    emp = rng.uniform(-0.3, 0.9, (4, nkp))
    enk = np.concatenate([core, np.sort(occ, axis=0), np.sort(emp, axis=0)])
    out["offsets"] = dict(enk=np.asfortranarray(enk), ef=0.0, kqid=p.kqm.kqid[:, iq], ncg=1, nomx=2, numin=1,
                          omega=np.array([0.05, 0.5, 5.0]), tetc=p.kqm.tetc)
    # static limit: q = Γ (k - q = k), frequencies 0 and 1e-7 besides finite
    # ones, a band 1e-7 above the lowest one at half of the k-points (weights
    # beyond stweight_imag_par's unphysical-weight tolerance, zeroed below
    # |ω| = 1e-6), and one tetrahedron whose polyhedron has six nodes with
    # two quadrilateral faces (sortnodes' two-square branch)
    rng = np.random.default_rng(0)
    occ = rng.uniform(-0.6, 0.4, (3, nkp))
    emp = rng.uniform(-0.3, 0.9, (2, nkp))
    near = occ[:1] + 1e-7 * rng.choice([0.0, 1.0], (1, nkp))
    enk = np.concatenate([occ, near, emp])
    c0 = p.kqm.tetc[:, 0]
    enk[0, c0] = [-1.0, -0.25, 0.5, -0.5]
    enk[4, c0] = [0.5, 0.0, -0.25, 0.75]
    out["static"] = dict(enk=np.asfortranarray(enk), ef=0.0, kqid=np.arange(nkp), ncg=0, nomx=2, numin=0,
                         omega=np.array([0.0, 1e-7, 1e-3, 0.5, 5.0]), tetc=p.kqm.tetc)
    return out


def check_full_c1():
    """Optional (--check-c1, nothing stored, about ten minutes): the full C1
    problem (3³ k, 16 × 28 band pairs, four frequencies, the last q) through
    the reference's statements and through the oracle with the reference's
    wtemp addressing; prints how many of the kcw entries differ."""
    from oracle import weights as ow
    from pygw_gb300 import synthetic as syn
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, nom=4)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    args = (b.enk(), b.EF, p.kqm.kqid[:, p.qs[-1]], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    portable = (lambda x: float(ow.portable_math(np.array([x]))[0][0]),
                lambda x: float(ow.portable_math(np.array([x]))[1][0]))
    ref = reference_par2(portable)(*args)
    with ow.reference_layout():
        got = ow.bz_calcqdepw_par2(*args)
    print(f"full C1: kcw {ref.shape}, {np.count_nonzero(ref)} nonzero, "
          f"{np.count_nonzero(got != ref)} entries differ from the reference's statements")


def main():
    from oracle import weights as ow
    if "--check-c1" in sys.argv:
        check_full_c1()
        return

    def portable_atan(x):
        return float(ow.portable_math(np.array([x]))[0][0])

    def portable_log(x):
        return float(ow.portable_math(np.array([x]))[1][0])

    variants = {"libm": (math.atan, math.log), "portable": (portable_atan, portable_log)}
    store = {}
    rng = np.random.default_rng(2)
    for name, c in cases().items():
        # an SVD frequency basis for bz_calcqdepw_par3: dUl[nom, nl]
        c["dUl"] = rng.standard_normal((len(c["omega"]), 3))
        for k, v in c.items():
            store[f"{name}.{k}"] = np.asarray(v)
        for vname, impl in variants.items():
            run = reference_par2(impl)
            kcw = run(c["enk"], c["ef"], c["kqid"], c["ncg"], c["nomx"], c["numin"], c["omega"], c["tetc"])
            store[f"{name}.kcw_{vname}"] = kcw
            print(f"{name} ({vname}): kcw {kcw.shape}, {np.count_nonzero(kcw)} nonzero", flush=True)
            run3 = reference_par3(impl)
            kcw3 = run3(c["enk"], c["ef"], c["kqid"], c["ncg"], c["nomx"], c["numin"], c["dUl"], c["omega"],
                        c["tetc"])
            store[f"{name}.kcw3_{vname}"] = kcw3
            print(f"{name} ({vname}): par3 kcw {kcw3.shape}", flush=True)
    np.savez_compressed(OUT, **store)
    print("wrote", OUT)


if __name__ == "__main__":
    refsrc.run(main)
