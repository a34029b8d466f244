"""The numpy oracle of calc_eps against golden vectors from the reference's own
calc_eps (pygw.py:3039-3297), run on seeded inputs by
tests/golden/make_calc_eps_golden.py: a finite q, q = 0 with head and wings,
q = 0 in an SVD frequency basis, and q = 0 with core states.  Both sides are FP64 numpy; only the
order of some sums differs, so the bar is 1e-12 of the largest entry.  The
GPU paths are checked against this oracle (tests/test_gpu_*.py)."""
import os

import numpy as np
import pytest

from oracle import eps as oe

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "calc_eps_golden.npz"))


def _g(case, key):
    return GOLDEN[f"{case}.{key}"]


def _close(got, ref, tol=1e-12):
    return np.abs(np.asarray(got) - ref).max() <= tol * max(np.abs(ref).max(), 1e-300)


@pytest.mark.parametrize("case", ["q", "q0", "q0svd", "q0core"])
def test_oracle_calc_eps_matches_the_reference_code(case):
    M, kcw = _g(case, "M"), _g(case, "kcw")
    npb = M.shape[-1]
    q0 = case != "q"
    svd = case == "q0svd"
    pm = _g(case, "pm") if q0 else None
    eps, w1, w2, head, _ = oe.calc_eps(kcw, lambda ik: M[ik], npb,
                                       pm_k=(lambda ik: pm[ik]) if q0 else None,
                                       head=_g(case, "head_in") if q0 else None,
                                       Ul=_g(case, "Ul") if svd else None, dUl=_g(case, "dUl") if svd else None)
    assert eps.shape == _g(case, "eps").shape
    assert _close(eps, _g(case, "eps"))
    if q0:
        assert _close(w1, _g(case, "epsw1"))
        assert _close(w2, _g(case, "epsw2"))
        assert _close(head, _g(case, "head"))


@pytest.mark.parametrize("case", ["q0", "q0svd", "q0core"])
def test_product_momentum_vectors_match_the_reference_code(case):
    """The product's host-side q→0 vectors (eps.momentum_vectors), formed from
    the reference's head_quantities (momentum elements stored from band mst,
    core levels first; pygw.py:3089-3093, 3120-3141), equal the vectors the
    oracle above reproduces the reference's wings with, bit for bit."""
    from types import SimpleNamespace as NS

    from pygw_gb300 import eps as peps
    g = lambda k: _g(case, k)  # noqa: E731
    nkp = g("M").shape[0]
    ecore = g("ecore")
    ncg = len(ecore)
    nvbm1, ncbm = (int(x) for x in g("nomax_numin"))
    Ebnd = g("Ebnd")
    ks = NS(nomax_numin=(nvbm1, ncbm), ncg_p=ncg, nbmaxpol=Ebnd.shape[2], Ebnd=Ebnd)
    core = NS(corind=np.array([[0, 0, ic] for ic in range(ncg)], dtype=int).reshape(ncg, 3),
              eig_core=[[list(ecore)]])
    kqm = NS(kii_ind=np.arange(nkp))
    hq = (g("head_in"), g("mmatcv"), g("mmatvv"), int(g("mst")))
    pm = peps.momentum_vectors(hq, ks, core, kqm, float(g("Vol")))
    assert pm.shape == g("pm").shape
    assert np.array_equal(pm, g("pm"))
    assert np.count_nonzero(pm) == pm.size


def test_drop_in_calc_eps_forms_the_q0_vectors_from_head_quantities(monkeypatch):
    """MatrixElements2Band.calc_eps at q = 0 with the reference's arguments
    hands the contraction the reference's q→0 vectors and head (the GPU call
    itself is replaced by a recorder here)."""
    from types import SimpleNamespace as NS

    from pygw_gb300 import eps as peps
    case = "q0core"
    g = lambda k: _g(case, k)  # noqa: E731
    M, kcw = g("M"), g("kcw")
    nkp, nb1, nb2, npb = M.shape
    ecore = g("ecore")
    ncg = len(ecore)
    seen = {}

    def recorder(kcw_, minm, nkp_, npb_, nb1_, nb2_, nom_, pm_k=None, head=None, Ul=None, dUl=None):
        seen.update(pm=np.stack([pm_k(ik) for ik in range(nkp_)]), head=head, shape=(nkp_, npb_, nb1_, nb2_, nom_),
                    minm=np.stack([minm(ik) for ik in range(nkp_)]))
        z = np.zeros((npb_, npb_, nom_), complex)
        return NS(numpy=lambda: (z, None, None, None))

    monkeypatch.setattr(peps, "chi0_eps", recorder)
    nvbm1, ncbm = (int(x) for x in g("nomax_numin"))
    Ebnd = g("Ebnd")
    ks = NS(nomax_numin=(nvbm1, ncbm), ncg_p=ncg, nbmaxpol=Ebnd.shape[2], Ebnd=Ebnd)
    core = NS(corind=np.array([[0, 0, ic] for ic in range(ncg)], dtype=int).reshape(ncg, 3),
              eig_core=[[list(ecore)]])
    kqm = NS(kii_ind=np.arange(nkp))
    me = peps.MatrixElements2Band(lambda ik, iq, bl, mode: (M[ik][ncg:], M[ik][:ncg]), npb)
    hq = (g("head_in"), g("mmatcv"), g("mmatvv"), int(g("mst")))
    me.calc_eps(0, hq, None, None, NS(Vol=float(g("Vol"))), kqm, ks, None, None, None, core, None,
                NS(omega=np.zeros(kcw.shape[3])), kcw, "", None, None, None)
    assert seen["shape"] == (nkp, npb, nb1, nb2, kcw.shape[3])
    assert np.array_equal(seen["pm"], g("pm")) and np.array_equal(seen["head"], g("head_in"))
    assert np.array_equal(seen["minm"], M)            # core block first, as calc_eps concatenates
