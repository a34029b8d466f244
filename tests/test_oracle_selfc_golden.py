"""The self-energy oracle and the product's host glue against golden vectors
from the reference's own calc_selfc (pygw.py:3299-3412) and
Compute_selfc_inside (mcommon.py:80-165), run on seeded inputs by
tests/golden/make_calc_selfc_golden.py:

* mwm for a finite q and for q = 0 with the head and wing terms;
* the energies at k − q, core states first, against the product's helper;
* the convolutions of the plain, the iopfreq 4 (spline interpolation onto the
  dense mesh, of complex and of real mwm) and the SVD branches, with the reference's Fortran kernels
  (fnc.f90) run from their source text by the generator (tests/golden/f90py.py)
  — the golden values are the reference's own statements end to end.
"""
import os

import numpy as np
import pytest

from oracle import selfc as osc

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "calc_selfc_golden.npz"))
IBGW, NCG_C = 1, 1          # the generator's band window: GW bands 1..2, one core state
NCG = {"densereal": 0}      # cases without the core state


def _g(case, key):
    return GOLDEN[f"{case}.{key}"]


def _close(got, ref, tol=1e-12):
    return np.abs(np.asarray(got) - ref).max() <= tol * max(np.abs(ref).max(), 1e-300)


@pytest.mark.parametrize("case", ["q", "q0dense", "svd", "densereal"])
def test_oracle_mwm_matches_the_reference_code(case):
    M, W, wkq = _g(case, "M"), _g(case, "W"), float(_g(case, "wkq"))
    q0 = None
    if case == "q0dense":
        c1, c2 = _g(case, "coefs")
        q0 = (_g(case, "head"), _g(case, "epsw1"), _g(case, "epsw2"), c1, c2, NCG_C, IBGW)
    for ik in range(M.shape[0]):
        assert _close(osc.mwm_k(M[ik], W, wkq, q0=q0), _g(case, "mwm")[ik])


@pytest.mark.parametrize("case", ["q", "q0dense", "svd", "densereal"])
def test_energies_at_k_minus_q_match_the_reference_code(case):
    from pygw_gb300.selfc import _selfc_enk

    class Core:
        corind = np.array([[0, 0, 0]])
        eig_core = [[list(_g(case, "core_e"))]]
    iq = 0 if case == "q0dense" else 1
    Ebnd, kqid, enk = _g(case, "Ebnd"), _g(case, "kqid"), _g(case, "enk")
    for ik in range(enk.shape[0]):
        assert np.array_equal(_selfc_enk(Ebnd[0], NCG.get(case, NCG_C), Core, kqid[ik, iq], enk.shape[1]), enk[ik])


@pytest.mark.parametrize("c", ["q0dense", "densereal"])
def test_oracle_dense_mesh_branch_matches_the_reference_code(c):
    """Spline interpolation onto the dense mesh (mcommon.py:123-141); with W
    Hermitian (densereal) mwm is real up to rounding, and the reference, like
    the oracle, splines only its real part."""
    mean_im = np.abs(_g(c, "mwm").imag).mean(axis=1)
    assert (mean_im < 1e-10).all() if c == "densereal" else (mean_im > 1e-10).all()
    for ik in range(_g(c, "enk").shape[0]):
        sc = osc.interp_fr_convolutions(_g(c, "enk")[ik], _g(c, "mwm")[ik], _g(c, "omega"), _g(c, "omega_p"),
                                        _g(c, "womeg_p"))
        assert _close(sc, _g(c, "sc_p")[ik])


def test_oracle_svd_branch_matches_the_reference_code():
    c = "svd"
    for ik in range(_g(c, "enk").shape[0]):
        sc = osc.svd_fr_convolutions(_g(c, "enk")[ik], _g(c, "mwm")[ik], _g(c, "Ul"), _g(c, "omega"), _g(c, "womeg"))
        assert _close(sc, _g(c, "sc_p")[ik])
