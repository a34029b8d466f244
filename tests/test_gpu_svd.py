"""SVD frequency basis on the GPU: par3 weights against the oracle's par3, the
basis change, and calc_eps in SVD mode (FP64 and mixed precision, q ≠ 0 and
q → 0) against the oracle's SVD-mode calc_eps."""
import numpy as np
import pytest
import torch

from oracle import eps as oe
from oracle import weights as ow
from pygw_gb300 import eps as peps
from pygw_gb300 import svd
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _basis(nom, cutoff=1e-6):
    om, dom = svd.tan_mesh(0.02, 20.0, nom)
    return om[nom:], svd.svd_functions(om[nom:], dom[nom:], 0.01, 50.0, 200, cutoff)


def test_par3_weights_match_oracle():
    w = syn.scaled(syn.WORKLOADS["C1"], nom=24)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    om, (Ul, dUl) = _basis(24)
    for iq in p.qs[:1] + [0]:
        ref = ow.bz_calcqdepw_par3(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, dUl, om, p.kqm.tetc)
        got = svd.bz_calcqdepw_par3(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, dUl, om, p.kqm.tetc)
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_basis_change_matches_numpy():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(7, 33, 5)) + 1j * rng.normal(size=(7, 33, 5))
    U = rng.normal(size=(7, 11))
    y = svd.to_basis(torch.from_numpy(x).cuda(), U).cpu().numpy()
    assert np.max(np.abs(y - np.einsum("iab,ij->jab", x, U))) < 1e-13 * np.max(np.abs(y))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-9)])
def test_svd_calc_eps_matches_oracle(precision, tol):
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=96, nom=20)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    om, (Ul, dUl) = _basis(20)
    nl = Ul.shape[0]
    for iq in (p.qs[0], 0):
        kcw = ow.bz_calcqdepw_par3(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, dUl, om, p.kqm.tetc)
        sqv = syn.coulomb_sqrt(w, iq, w.npb)
        minm = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in range(p.kqm.nkp)]
        pm_k = head = None
        if iq == 0:
            pms = [syn.pm_k(w, b, ik) for ik in range(p.kqm.nkp)]
            pm_k = lambda ik: pms[ik]
            head = syn.head_from_weights(kcw, pms)          # in the basis, as calc_head returns it
        ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb, pm_k=pm_k, head=head, Ul=Ul, dUl=dUl)
        r = peps.chi0_eps(kcw, lambda ik: minm[ik], p.kqm.nkp, w.npb, b.nb1, b.nb2, nl, pm_k=pm_k, head=head,
                          precision=precision, Ul=Ul, dUl=dUl)
        got = r.numpy()
        assert got[0].shape == (w.npb, w.npb, nl)
        assert np.max(np.abs(got[0] - ref[0])) <= tol * np.max(np.abs(ref[0]))
        if iq == 0:
            for a, e in zip(got[1:], ref[1:4]):
                assert np.max(np.abs(a - e)) <= tol * max(1.0, np.max(np.abs(e)))


@pytest.mark.parametrize("name", ["c1", "stress"])
def test_par3_against_the_reference_statements(name):
    """The GPU par3 weights against kcw from the reference's own Fortran
    statements (tests/golden/weights_golden.npz, portable atan/log), within
    the GPU-vs-oracle par3 bar, outside the entries of 7- and 8-node items
    (the reference's wtemp layout aliases their frequencies, which the
    projection mixes into every basis function; see
    tests/test_oracle_weights_golden.py)."""
    from test_oracle_weights_golden import alias_mask, item_nodes, load_case
    a, ref = load_case(name, par=3)
    got = svd.bz_calcqdepw_par3(a["enk"], a["ef"], a["kqid"], a["ncg"], a["nomx"], a["numin"], a["dUl"], a["omega"],
                                a["tetc"])
    want = ref["portable"]
    assert got.shape == want.shape
    keep = ~alias_mask(a, item_nodes(a), par=3)
    assert np.max(np.abs(got - want)[keep]) <= 1e-13 * np.max(np.abs(want))


@pytest.mark.parametrize("name", ["c1", "stress"])
def test_par3_reference_layout_against_the_reference_statements(name):
    """par3 with the reference's wtemp addressing reproduced: within the
    GPU-vs-oracle par3 bar of the reference's statements at every entry."""
    from pygw_gb300 import polarization as pol
    from test_oracle_weights_golden import load_case
    a, ref = load_case(name, par=3)
    with pol.reference_layout():
        got = svd.bz_calcqdepw_par3(a["enk"], a["ef"], a["kqid"], a["ncg"], a["nomx"], a["numin"], a["dUl"],
                                    a["omega"], a["tetc"])
    want = ref["portable"]
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
