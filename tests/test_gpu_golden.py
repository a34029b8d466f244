"""The GPU ε path against golden vectors from the reference's own calc_eps
(pygw.py:3039-3297; tests/golden/make_calc_eps_golden.py): a finite q, q = 0
with head and wings, and q = 0 in an SVD frequency basis — through the
product's public call, in FP64 (1e-12 of the largest entry) and in split
precision (1e-9)."""
import os

import numpy as np
import pytest

from pygw_gb300 import eps as peps

pytestmark = pytest.mark.gpu

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "calc_eps_golden.npz"))


def _close(got, ref, tol):
    return np.abs(np.asarray(got) - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-9)])
@pytest.mark.parametrize("case", ["q", "q0", "q0svd"])
def test_gpu_calc_eps_matches_the_reference_code(case, precision, tol):
    g = lambda k: GOLDEN[f"{case}.{k}"]  # noqa: E731
    M, kcw = g("M"), g("kcw")
    nkp, nb1, nb2, npb = M.shape
    q0, svd = case != "q", case == "q0svd"
    pm = g("pm") if q0 else None
    r = peps.chi0_eps(kcw, lambda ik: M[ik], nkp, npb, nb1, nb2, kcw.shape[3],
                      pm_k=(lambda ik: pm[ik]) if q0 else None, head=g("head_in") if q0 else None,
                      precision=precision, Ul=g("Ul") if svd else None, dUl=g("dUl") if svd else None)
    eps, w1, w2, head = r.numpy()
    assert _close(eps, g("eps"), tol)
    if q0:
        assert _close(w1, g("epsw1"), tol) and _close(w2, g("epsw2"), tol) and _close(head, g("head"), tol)
