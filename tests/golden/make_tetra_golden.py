"""Generate golden single-tetrahedron weights from the reference's Fortran statements.

Run where the reference's source tree is available:

    python tests/golden/make_tetra_golden.py --reference <PyGW source tree>

The reference's ``convw1t_par`` (for_tetrahedra3.f90:3-136) and its callees
(``surfnodes``, ``unrepnodes``, ``relnodes``, ``sortnodes``: for_tetrahedra2.f90:
1803-2773; ``generictetra_par``, ``stweight_imag_par``, ``stweight_itaylor_par``:
for_tetrahedra3.f90:220-743; ``sorteq``: for_tetrahedra2.f90:1688-1798) are
executed from their Fortran text through ``f90py`` (beside this script) on one
tetrahedron at a time: corner energies e (occupied band) and f (empty band)
with EF = 0, at six imaginary frequencies that include 0 and 1e-7.  The
polyhedron {e <= EF < f} and the branch of ``sortnodes`` that orders its nodes
depend only on these eight numbers, so a population of seeded corner sets
reaches the geometric cases far more densely than band structures on a mesh:

* ``grid``: energies on a grid of 0.25 (corners on EF, equal corners, e = f);
* ``near``: f = e + {0, 1e-7, 1e-3, 0.25} (weights beyond the unphysical-weight
  tolerance, the ω -> 0 branches);
* ``cont``: continuous energies;
* ``equal``: f - e the same at all four corners (the polyhedron a slab, every
  sub-tetrahedron's corner differences equal), or all corners occupied and
  f - e apart by steps of 0.6 % (sorteq's groupings within its relative
  tolerance of 1e-2, including chains that are not transitive).

atan and log are the portable implementations the oracle and the GPU kernels
share; the well-defined sets are run once more with the C library's atan and
log (``weight_libm``).  Each tetrahedron is classified:

* 0 — the reference's statements run to the end; ``weight[4, nom]`` stored;
* 1 — they address outside an array's storage, test a bit outside an
  integer, or give weights that depend on a variable never written (run with
  ``f90py.POISON``: such reads give NaN or the integer type's lowest value):
  each undefined in compiled code;
* 2 — they call ``stop`` (also with ``POISON`` off: a stop reached only
  from poisoned values follows from storage never written and is class 1);
  ``stop_site`` records which one (``STOP_SITES``).

``--coverage`` stores nothing and instead lists, per translated routine, the
statements that no well-defined tetrahedron executes.  ``--search SEED
PER_KIND`` stores nothing and instead runs PER_KIND fresh corner sets of each
kind from SEED through the statements and through the oracle (with the
reference's layout of 7- and 8-node halves) and counts the sets where they
disagree: different weights, or a status that does not match the class.

Output: ``tetra_golden.npz`` (e, f, omega, kind, stop_site, weight and
weight_libm per tetrahedron); nothing of the reference's source is stored.
"""
import contextlib
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
import f90py  # noqa: E402
from refsrc import reference_file  # noqa: E402

OUT = os.path.join(HERE, "tetra_golden.npz")
FILES = ["for_tetrahedra.f90", "for_tetrahedra2.f90", "for_tetrahedra3.f90"]
OMEGA = np.array([0.0, 1e-7, 1e-3, 0.05, 0.5, 5.0])
COUNTS = {"grid": 400, "near": 300, "cont": 200, "equal": 200}
# the stop messages of convw1t_par and its callees, by site code 1..
STOP_SITES = ["ERROR in sortnodes", "error in sortnodes, nnod=6", "error in setnodes", "ERROR in sorteq",
              "ERROR in convw1t", "ERROR in stweight_imat"]


def corner_sets(kind, n, rng):
    out = []
    for _ in range(n):
        if kind == "grid":
            e = np.round(rng.uniform(-1, 0.6, 4) * 4) / 4
            f = np.round(rng.uniform(-0.6, 1, 4) * 4) / 4
        elif kind == "near":
            e = np.round(rng.uniform(-1, 0.6, 4) * 4) / 4
            f = e + rng.choice([0.0, 1e-7, 1e-3, 0.25], 4) * rng.choice([-1, 1], 4)
        elif kind == "cont":
            e = rng.uniform(-1, 0.6, 4)
            f = rng.uniform(-0.6, 1, 4)
        elif rng.uniform() < 0.5:
            e = rng.uniform(-1, 0.6, 4)
            f = e + rng.uniform(0.3, 1.5)
        else:
            e = rng.uniform(-1, -0.1, 4)
            f = e + rng.uniform(0.3, 1.5) * (1 + 0.006 * rng.choice([0, 1, 2, 3, 5], 4))
        out.append((e + 0.0, f + 0.0))          # -0.0 -> 0.0
    return out


def main():
    from oracle import weights as ow

    def portable_atan(x):
        return float(ow.portable_math(np.array([x]))[0][0])

    def portable_log(x):
        return float(ow.portable_math(np.array([x]))[1][0])

    coverage = "--coverage" in sys.argv
    search = sys.argv.index("--search") if "--search" in sys.argv else None
    counts, seed = COUNTS, 7
    if search is not None:           # --search SEED PER_KIND: compare with the oracle, store nothing
        seed, per = int(sys.argv[search + 1]), int(sys.argv[search + 2])
        counts = {kind: per for kind in COUNTS}
    f90py.POISON = True
    procs, tr = f90py.load([reference_file(f) for f in FILES], ["convw1t_par"], portable_atan, portable_log)
    conv = procs["convw1t_par"]
    nom = len(OMEGA)
    rng = np.random.default_rng(seed)

    def call(e, f):
        w = f90py.FArr(np.zeros((4, nom), order="F"), (1, 1))
        conv(w, f90py.FArr(e.copy(), (1,)), f90py.FArr(f.copy(), (1,)), np.array(0.0),
             f90py.FArr(OMEGA.copy(), (1,)), np.array(nom, dtype=np.int32), np.array(False))
        return w

    def stop_site(ex):
        msg = str(ex).strip("'\" ")
        return STOP_SITES.index(msg) + 1

    E, F, K, S, W = [], [], [], [], []
    hits = {}
    for kind, n in counts.items():
        for e, f in corner_sets(kind, n, rng):
            trace = f90py.LineTrace() if coverage else contextlib.nullcontext()
            site = 0
            try:
                with trace:
                    w = call(e, f)
                k = 0 if np.isfinite(w.a).all() else 1
            except f90py.Undefined:
                k = 1
            except f90py.FortranStop:
                f90py.POISON = False              # does it stop from defined values too?
                try:
                    call(e, f)
                    k = 1
                except f90py.Undefined:
                    k = 1
                except f90py.FortranStop as ex:
                    k, site = 2, stop_site(ex)
                finally:
                    f90py.POISON = True
            if coverage and k == 0:
                for u, ls in trace.hits.items():
                    hits.setdefault(u, set()).update(ls)
            E.append(e)
            F.append(f)
            K.append(k)
            S.append(site)
            W.append(w.a.copy() if k == 0 else np.zeros((4, nom)))
        print(kind, n, "done", flush=True)
    if search is not None:
        bad = 0
        with ow.reference_layout():
            for e, f, k, site, w in zip(E, F, K, S, W):
                got, st, _ = ow.convw1t(e, f, 0.0, OMEGA)
                bad += bool((k == 0 and (st or not np.array_equal(got, w))) or (k == 1 and not st & 32)
                            or (k == 2 and (not st or st & 32)))
        print(f"{len(K)} corner sets (seed {seed}): {np.bincount(K, minlength=3).tolist()} defined / undefined / "
              f"stop; {bad} where the oracle disagrees")
        return
    if coverage:
        # statements the well-defined tetrahedra never execute
        for u, (n_run, n_all, miss) in f90py.unexecuted(tr, hits).items():
            print(f"{u}: {n_run}/{n_all} statements executed")
            for m in miss:
                print("    never:", m)
        return
    K = np.array(K, dtype=np.int8)
    # the well-defined sets once more with the C library's atan/log
    procs_libm, _ = f90py.load([reference_file(f) for f in FILES], ["convw1t_par"], math.atan, math.log)
    conv = procs_libm["convw1t_par"]
    WL = np.zeros((len(K), 4, nom))
    for i in np.flatnonzero(K == 0):
        WL[i] = call(E[i], F[i]).a
        assert np.isfinite(WL[i]).all()
    np.savez_compressed(OUT, e=np.array(E), f=np.array(F), omega=OMEGA, kind=K, weight=np.array(W),
                        weight_libm=WL, stop_site=np.array(S, dtype=np.int8))
    print("wrote", OUT, "kinds:", np.bincount(K, minlength=3).tolist())


if __name__ == "__main__":
    main()
