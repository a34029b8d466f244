"""The numpy restatement of calc_eps against closed forms and linear algebra (CPU)."""
import numpy as np

from oracle import eps as oe
from oracle import weights as ow
from pygw_gb300 import synthetic as syn


def _c1_small(npb=24, nbands=10, nocc=3):
    w = syn.scaled(syn.WORKLOADS["C1"], nbands=nbands, nocc=nocc, npb=npb, nom=6, div=3)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    sqv = syn.coulomb_sqrt(w, iq, npb)
    minm = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in range(p.kqm.nkp)]
    return p, kcw, minm


def test_contraction_equals_einsum():
    p, kcw, minm = _c1_small()
    npb = minm[0].shape[-1]
    eps, _, _, _, chi0 = oe.calc_eps(kcw, lambda ik: minm[ik], npb)
    nb1, nb2, nkp, nom = kcw.shape
    M = np.stack(minm)                                     # [k, nb1, nb2, I]
    ref = -2.0 * np.einsum("kabi,abkw,kabj->ijw", M, kcw, np.conj(M))
    assert np.max(np.abs(chi0 - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_dielectric_matrix_is_hermitian_positive_and_inverted():
    p, kcw, minm = _c1_small()
    npb = minm[0].shape[-1]
    eps, _, _, _, chi0 = oe.calc_eps(kcw, lambda ik: minm[ik], npb)
    for w in range(kcw.shape[-1]):
        e = (chi0[:, :, w] + chi0[:, :, w].conj().T) / 2 + np.eye(npb)
        ev = np.linalg.eigvalsh(e)
        assert ev.min() > 1 - 1e-2                  # ε = 1 + (≈PSD): eigenvalues ≥ 1 up to the weight approximations
        inv = eps[:, :, w] + np.eye(npb)
        assert np.max(np.abs(inv @ e - np.eye(npb))) < 1e-12


def test_flat_bands_constant_matrix_elements_closed_form():
    """Flat bands and k-independent M: χ0 = −2 Σ_p M_p M_pᴴ Σ_k w_p(k) with
    Σ_k w_p = −2Δ_p/(ω²+Δ_p²)."""
    w = syn.scaled(syn.WORKLOADS["C1"], nbands=5, nocc=2, jitter=0.0, t_hop=0.0, nom=5, div=3, om_hi=1.0)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, p.qs[0]], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    nb1, nb2 = kcw.shape[:2]
    rng = np.random.default_rng(5)
    npb = 7
    M = rng.standard_normal((nb1, nb2, npb)) + 1j * rng.standard_normal((nb1, nb2, npb))
    _, _, _, _, chi0 = oe.calc_eps(kcw, lambda ik: M, npb)
    enk = b.enk()
    ref = np.zeros((npb, npb, len(p.fr.omega)), complex)
    for ib in range(nb1):
        for jb in range(nb2):
            d = enk[numin + jb, 0] - enk[ib, 0]
            if enk[numin + jb, 0] <= b.EF:
                continue
            s = -2.0 * d / (p.fr.omega ** 2 + d ** 2)
            ref += -2.0 * np.outer(M[ib, jb], M[ib, jb].conj())[:, :, None] * s[None, None, :]
    assert np.max(np.abs(chi0 - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_q0_head_wings_update():
    """The q→0 update of pygw.py:3246-3263.  Its head is the Schur-complement
    inverse of the bordered matrix [[1+head, w1ᴴ], [w1, ε]]; its body update
    uses w2b = conj(ε⁻¹·conj(w1)) = (ε⁻¹)ᵀ·w1, i.e. the border w1ᵀ instead of
    w1ᴴ — the two agree only for real wings.  Both are checked as written."""
    p, kcw, minm = _c1_small()
    npb = minm[0].shape[-1]
    rng = np.random.default_rng(9)
    P = kcw.shape[0] * kcw.shape[1]
    pms = [(rng.standard_normal(P) + 1j * rng.standard_normal(P)) * 0.1 for _ in range(len(minm))]
    head0 = np.abs(rng.standard_normal(kcw.shape[-1])) + 0.5
    eps, w1, w2, head, chi0 = oe.calc_eps(kcw, lambda ik: minm[ik], npb, pm_k=lambda ik: pms[ik], head=head0)
    raw = np.zeros((npb, kcw.shape[-1]), complex)
    for ik in range(len(minm)):
        m2 = minm[ik].reshape(P, npb)
        for om in range(kcw.shape[-1]):
            raw[:, om] += (m2.T * -2.0 * kcw[:, :, ik, om].ravel()) @ pms[ik]
    for om in range(kcw.shape[-1]):
        body = (chi0[:, :, om] + chi0[:, :, om].conj().T) / 2 + np.eye(npb)
        big = np.zeros((npb + 1, npb + 1), complex)
        big[0, 0] = 1 + head0[om]
        big[0, 1:] = np.conj(raw[:, om])
        big[1:, 0] = raw[:, om]
        big[1:, 1:] = body
        inv = np.linalg.inv(big)
        np.testing.assert_allclose(head[om] + 1, inv[0, 0], rtol=1e-10)
        binv = np.linalg.inv(body)
        h = inv[0, 0]
        bw1 = binv @ raw[:, om]
        w2b = np.conj(binv) @ raw[:, om]
        np.testing.assert_allclose(eps[:, :, om] + np.eye(npb), binv + h * np.outer(bw1, w2b), rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(w1[:, om], -h * bw1, rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(w2[:, om], -h * w2b, rtol=1e-9, atol=1e-14)
