"""The numpy oracle of calc_eps against golden vectors from the reference's own
calc_eps (pygw.py:3039-3297), run on seeded inputs by
tests/golden/make_calc_eps_golden.py: a finite q, q = 0 with head and wings,
and q = 0 in an SVD frequency basis.  Both sides are FP64 numpy; only the
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


@pytest.mark.parametrize("case", ["q", "q0", "q0svd"])
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
