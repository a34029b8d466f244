"""SVD frequency basis (iopfreq = 5): basis construction and the oracle's par3
weights and SVD-mode calc_eps, checked by identities that need no GPU."""
import numpy as np

from oracle import eps as oe
from oracle import weights as ow
from pygw_gb300 import svd
from pygw_gb300 import synthetic as syn


def _mats(nom, cutoff):
    om, dom = svd.tan_mesh(0.02, 20.0, nom)
    return om[nom:], dom[nom:], svd.svd_functions(om[nom:], dom[nom:], 0.01, 50.0, 200, cutoff)


def test_basis_is_a_left_inverse_pair():
    iw, wiw, (Ul, dUl) = _mats(32, 1e-6)
    nl = Ul.shape[0]
    assert Ul.shape == (nl, 32) and dUl.shape == (32, nl) and 4 < nl < 32
    assert np.max(np.abs(Ul @ dUl - np.eye(nl))) < 1e-8
    # positive frequencies in ascending order
    assert np.all(np.diff(iw) > 0) and iw[0] > 0


def test_par3_is_par2_projected():
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, nom=12)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    _, _, (Ul, dUl) = _mats(12, 1e-6)
    iq = p.qs[0]
    k2 = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    k3 = ow.bz_calcqdepw_par3(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, dUl, p.fr.omega, p.kqm.tetc)
    ref = np.einsum("abkw,wl->abkl", k2, dUl)
    assert np.max(np.abs(k3 - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_svd_calc_eps_with_a_complete_basis_equals_the_projected_plain_result():
    # square basis: dUl·Ul = I, so the SVD flow is the plain flow followed by ·dUl
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, nom=6, npb=24)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    rng = np.random.default_rng(0)
    dUl = np.linalg.qr(rng.normal(size=(6, 6)))[0]
    Ul = np.linalg.inv(dUl)
    k2 = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    k3 = np.einsum("abkw,wl->abkl", k2, dUl)
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    minm = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in range(p.kqm.nkp)]
    plain = oe.calc_eps(k2, lambda ik: minm[ik], w.npb)[0]
    svdr = oe.calc_eps(k3, lambda ik: minm[ik], w.npb, Ul=Ul, dUl=dUl)[0]
    assert np.max(np.abs(svdr - np.dot(plain, dUl))) < 1e-12 * np.max(np.abs(plain))
