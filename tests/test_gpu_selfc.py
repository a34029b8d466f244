"""calc_selfc on the GPU against the oracle: the mwm contraction (FP64 and
split precision), its q = 0 terms, the three Matsubara convolutions, and the
drop-in calc_selfc end to end."""
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from oracle import selfc as osc
from pygw_gb300 import selfc as gsc

pytestmark = pytest.mark.gpu


def _crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _case(seed, nk=3, nb1=4, nb2=11, N=300, nom=5):
    rng = np.random.default_rng(seed)
    M = _crandn(rng, nk, nb1, nb2, N) / (1.0 + rng.uniform(0, 3, size=(nk, nb1, nb2, 1)))
    W = _crandn(rng, N, N, nom) * 0.05
    for w in range(nom):                                   # ε⁻¹ − 1 is Hermitian on the imaginary axis
        W[:, :, w] = 0.5 * (W[:, :, w] + W[:, :, w].conj().T) - 0.3 * np.eye(N)
    return M, W


def _normwise(got, want, M, W, wkq):
    """max_p |Δ mwm| / (wkq·‖M_p‖²·max_ω ‖W_ω‖_2): the error relative to the bound of |M_pᴴ W M_p|."""
    nk, nb1, nb2, N = M.shape
    wn = max(np.linalg.norm(W[:, :, w], 2) for w in range(W.shape[2]))
    m2 = np.sum(np.abs(M) ** 2, axis=-1).reshape(nk, 1, nb1 * nb2)
    return float(np.max(np.abs(got - want) / (wkq * m2 * wn)))


def _oracle_mwm(M, W, wkq, q0=None):
    nk, nb1, nb2, _ = M.shape
    return np.stack([osc.mwm_k(M[k], W, wkq, q0).reshape(W.shape[2], nb1 * nb2) for k in range(nk)])


@pytest.mark.parametrize("precision,omega_batch", [("fp64", None), ("mixed", None), ("mixed", 2)])
def test_mwm_matches_oracle(precision, omega_batch):
    M, W = _case(11)
    nk, nb1, nb2, N = M.shape
    wkq = 1.0 / 27
    got = gsc.mwm(M, W, nb1, nb2, wkq, precision=precision, omega_batch=omega_batch).cpu().numpy()
    want = _oracle_mwm(M, W, wkq)
    err = _normwise(got, want, M, W, wkq)
    rel = float(np.max(np.abs(got - want)) / np.max(np.abs(want)))
    print(f"mwm {precision} batch={omega_batch}: normwise {err:.3e}, max-relative {rel:.3e}")
    if precision == "fp64":
        assert err < 1e-14 and rel < 1e-12
    else:
        # five 8-bit digits: each product term is exact to ≈ 2^-40 of its row and column scales
        assert err < 1e-10 and rel < 1e-9


def test_mwm_mixed_ragged_sizes():
    # R = nk·P and N off every tile multiple; one k-point
    M, W = _case(12, nk=1, nb1=3, nb2=7, N=131, nom=3)
    nk, nb1, nb2, N = M.shape
    got = gsc.mwm(M, W, nb1, nb2, 0.5, precision="mixed").cpu().numpy()
    want = _oracle_mwm(M, W, 0.5)
    assert _normwise(got, want, M, W, 0.5) < 1e-10


def test_mwm_q0_terms():
    M, W = _case(13, nk=2, nb1=3, nb2=9, N=64, nom=4)
    nk, nb1, nb2, N = M.shape
    rng = np.random.default_rng(14)
    head = _crandn(rng, 4)
    w1, w2 = _crandn(rng, N, 4), _crandn(rng, N, 4)
    ibgw, ncg = 1, 2
    out = gsc.mwm(M, W, nb1, nb2, 0.25, precision="fp64")
    gsc.mwm_q0(out, M, nb1, nb2, ibgw + ncg, head, w1, w2, 0.7, 1.3)
    want = _oracle_mwm(M, W, 0.25, q0=(head, w1, w2, 0.7, 1.3, ncg, ibgw))
    got = out.cpu().numpy()
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))


def _conv_case(seed, nk=2, nb1=3, nb2=7, nom=12):
    rng = np.random.default_rng(seed)
    om = np.geomspace(0.01, 50.0, nom)
    wom = np.gradient(om)
    mwm = _crandn(rng, nk, nom, nb1 * nb2) / (1 + om[None, :, None] ** 2)
    mwm[0, :, 2] = 0.0                   # |mwm_iom| ≤ 1e-16: no arctan term
    mwm[1, :, 5] = mwm[1, :, 5].real     # a real row (dropped imaginary part in the spline branch)
    mwm[1, :, 6] = mwm[1, :, 6].real + 1e-13j
    enk = rng.uniform(-2.0, 2.0, size=(nk, nb2))
    return om, wom, mwm, enk


def test_convolution_matches_oracle():
    om, wom, mwm, enk = _conv_case(21)
    nk, nom, P = mwm.shape
    nb1, nb2 = 3, 7
    got = gsc.convolution(torch.from_numpy(mwm).cuda(), enk, om, wom, nb1, nb2).cpu().numpy()
    for k in range(nk):
        want = osc.all_fr_convolutions(enk[k], mwm[k].reshape(nom, nb1, nb2), om, wom)
        assert np.max(np.abs(got[k] - want)) <= 1e-12 * np.max(np.abs(want))


def test_convolution_dense_mesh_matches_oracle():
    pytest.importorskip("scipy")
    om, wom, mwm, enk = _conv_case(22)
    nk, nom, P = mwm.shape
    nb1, nb2 = 3, 7
    omd = np.geomspace(0.005, 80.0, 150)         # denser (two slices of the kernel's 128-point tile), beyond both ends
    womd = np.gradient(omd)
    got = gsc.convolution(torch.from_numpy(mwm).cuda(), enk, om, wom, nb1, nb2, dense=(omd, womd)).cpu().numpy()
    for k in range(nk):
        want = osc.interp_fr_convolutions(enk[k], mwm[k].reshape(nom, nb1, nb2), om, omd, womd)
        err = np.max(np.abs(got[k] - want)) / np.max(np.abs(want))
        assert err <= 1e-11, err


def test_convolution_svd_matches_oracle():
    rng = np.random.default_rng(23)
    nk, nb1, nb2, nl, nom = 2, 3, 6, 4, 10
    om = np.geomspace(0.02, 40.0, nom)
    wom = np.gradient(om)
    # basis functions decay with ω like the SVD functions of the bosonic kernel; random ones that
    # do not would make the terms near ω_i ≈ ω large against their sum
    Ul = rng.standard_normal((nl, nom)) / (1.0 + om[None, :] ** 2) + 0j
    mwm = _crandn(rng, nk, nl, nb1 * nb2)
    enk = rng.uniform(-2.0, 2.0, size=(nk, nb2))
    got = gsc.convolution(torch.from_numpy(mwm).cuda(), enk, om, wom, nb1, nb2, Ul=Ul).cpu().numpy()
    for k in range(nk):
        want = osc.svd_fr_convolutions(enk[k], mwm[k].reshape(nl, nb1, nb2), Ul, om, wom)
        assert np.max(np.abs(got[k] - want)) <= 1e-12 * np.max(np.abs(want))


def _selfc_problem(N=96, nom=6):
    """A tiny q = 0 problem with the objects calc_selfc reads."""
    rng = np.random.default_rng(31)
    nirk, nkp = 3, 4
    ncg, nbands, ibgw, nbgw = 2, 9, 1, 4
    ks = SimpleNamespace(ibgw=ibgw, nbgw=nbgw, ncg_c=ncg, nbands_c=nbands,
                         Ebnd=rng.uniform(-1.5, 2.5, size=(1, nirk, nbands + 3)))
    kqm = SimpleNamespace(weight=np.ones(nirk), k_ind=np.array([0, 1, 3]), kqid=np.array([[0], [2], [1], [3]]),
                          kii_ind=np.array([0, 1, 2, 1]), qlist=np.zeros((nkp, 3)))
    core = SimpleNamespace(corind=np.array([[0, 0, 0], [0, 0, 1]]), eig_core=[[np.array([-20.0, -12.5])]])
    om = np.geomspace(0.02, 30.0, nom)
    fr = SimpleNamespace(omega=om, womeg=np.gradient(om), iopfreq=3)
    latgen = SimpleNamespace(Vol=150.0)
    nb1 = nbgw - ibgw
    mins = {ik: (_crandn(rng, nb1, nbands - ncg, N) * 0.3, _crandn(rng, nb1, ncg, N) * 0.1) for ik in range(nkp)}

    def calc_minm(ik, iq, band_limits, mode, *rest):
        assert mode == "selfe" and band_limits == (ibgw, nbgw, 0, nbands - ncg, 0, ncg)
        return mins[ik]
    W = _crandn(rng, N, N, nom) * 0.05
    for w in range(nom):
        W[:, :, w] = 0.5 * (W[:, :, w] + W[:, :, w].conj().T) - 0.4 * np.eye(N)
    head = rng.uniform(-0.5, -0.1, nom) + 0j
    w1 = _crandn(rng, N, nom) * 0.1
    w2 = np.conj(w1)
    return ks, kqm, core, fr, latgen, calc_minm, mins, W, head, w1, w2


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-9)])
def test_calc_selfc_dropin(precision, tol):
    from pygw_gb300 import eps as geps
    ks, kqm, core, fr, latgen, calc_minm, mins, W, head, w1, w2 = _selfc_problem()
    N = W.shape[0]
    me = geps.MatrixElements2Band(calc_minm, N, singc1=0.35, singc2=1.7)
    old = geps.PRECISION
    geps.PRECISION = precision
    try:
        got = me.calc_selfc(0, W, w1, w2, head, None, None, latgen, kqm, ks, None, None, None, core, None, fr, None,
                            None, None, None)
    finally:
        geps.PRECISION = old
    # oracle: the reference's loop (pygw.py:3335-3385) with the restated pieces
    coefs2 = 1.7 * 4 * np.pi / latgen.Vol
    coefs1 = 0.35 * np.sqrt(4 * np.pi / latgen.Vol)
    wkq = 1.0 / len(kqm.qlist)
    for irk in range(len(kqm.weight)):
        ik = kqm.k_ind[irk]
        jrk = kqm.kii_ind[kqm.kqid[ik, 0]]
        minm = np.concatenate((mins[ik][1], mins[ik][0]), axis=1)
        mwm = osc.mwm_k(minm, W, wkq, q0=(head, w1, w2, coefs1, coefs2, ks.ncg_c, ks.ibgw))
        enk = np.concatenate(([-20.0, -12.5], ks.Ebnd[0, jrk, :ks.nbands_c - ks.ncg_c]))
        want = osc.all_fr_convolutions(enk, mwm, fr.omega, fr.womeg)
        err = np.max(np.abs(got[irk] - want)) / np.max(np.abs(want))
        print(f"calc_selfc {precision} irk={irk}: {err:.3e}")
        assert err <= tol
