"""The SVD frequency basis of the product (pygw_gb300.svd) against golden
vectors from the reference's own svd_functions (pygw.py:3478-3501) and
Give2TanMesh (mcommon.py:13-31), run on three Matsubara meshes (one with a
lower bound that Give2TanMesh clamps) by
tests/golden/make_svd_golden.py.  Both use scipy's SVD; a singular vector is
compared up to its sign."""
import os

import numpy as np
import pytest

from pygw_gb300 import svd

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "svd_golden.npz"))


@pytest.mark.parametrize("case", ["a", "b", "c"])
def test_svd_basis_matches_the_reference_code(case):
    g = lambda k: GOLDEN[f"{case}.{k}"]  # noqa: E731
    om_min, om_max, om_nom, cut = g("args")
    om, dom = svd.tan_mesh(om_min, om_max, int(om_nom))
    assert np.allclose(om, g("om"), rtol=1e-13, atol=0) and np.allclose(dom, g("dom"), rtol=1e-13, atol=0)
    Ul, dUl = svd.svd_functions(g("iomega"), g("wiomeg"), om_min, om_max, int(om_nom), cut)
    assert Ul.shape == g("Ul").shape and dUl.shape == g("dUl").shape
    sign = np.sign(np.sum(Ul * g("Ul"), axis=1))
    assert np.abs(sign[:, None] * Ul - g("Ul")).max() <= 1e-10 * np.abs(g("Ul")).max()
    assert np.abs(dUl * sign[None, :] - g("dUl")).max() <= 1e-10 * np.abs(g("dUl")).max()
