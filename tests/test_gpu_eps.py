"""GPU χ0 contraction and ε⁻¹ (plain FP64 path) vs the numpy restatement.

Tolerance: 1e-12 relative to the largest magnitude of each compared array —
the FP64 sums differ from numpy's BLAS only in summation order.
"""
import numpy as np
import pytest
import torch

from oracle import eps as oe
from oracle import weights as ow
from pygw_gb300 import eps as peps
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _problem(name="C1", **kw):
    w = syn.scaled(syn.WORKLOADS[name], **kw) if kw else syn.WORKLOADS[name]
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    minm = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in range(p.kqm.nkp)]
    return w, p, kcw, minm


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_chi0_fp64_matches_oracle():
    w, p, kcw, minm = _problem()
    nb1, nb2, nkp, nom = kcw.shape
    ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb)
    eps, _ = peps.chi0_accumulate(peps._kcw_device(kcw), lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom, k_chunk=5)
    peps.chi0_finalize(eps, w.npb, nom)
    chi0 = eps.cpu().numpy().transpose(2, 1, 0)
    chi0_ref = ref[4]
    herm_ref = (chi0_ref + np.conj(chi0_ref.transpose(1, 0, 2))) / 2
    assert _rel(chi0, herm_ref) < TOL


def test_eps_inverse_fp64_matches_oracle():
    w, p, kcw, minm = _problem()
    nb1, nb2, nkp, nom = kcw.shape
    ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb)
    r = peps.chi0_eps(kcw, lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom, k_chunk=8)
    eps = r.numpy()[0]
    for om in range(nom):
        assert _rel(eps[:, :, om] + np.eye(w.npb), ref[0][:, :, om] + np.eye(w.npb)) < TOL


def test_q0_head_and_wings_fp64():
    w, p, kcw, minm = _problem(div=3, npb=96, nom=8)
    nb1, nb2, nkp, nom = kcw.shape
    pms = [syn.pm_k(w, p.bands, ik) for ik in range(nkp)]
    head0 = syn.head_from_weights(kcw, pms)
    ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb, pm_k=lambda ik: pms[ik], head=head0)
    r = peps.chi0_eps(kcw, lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom, pm_k=lambda ik: pms[ik], head=head0)
    eps, w1, w2, head = r.numpy()
    assert _rel(head, ref[3]) < TOL
    assert _rel(w1, ref[1]) < 1e-11 and _rel(w2, ref[2]) < 1e-11
    for om in range(nom):
        assert _rel(eps[:, :, om] + np.eye(w.npb), ref[0][:, :, om] + np.eye(w.npb)) < 1e-11


def test_drop_in_calc_eps():
    w, p, kcw, minm = _problem(div=3, npb=64, nom=6)
    sqv = syn.coulomb_sqrt(w, p.qs[0], w.npb)

    def calc_minm(ik, iq, band_limits, mode):
        return syn.minm_k(w, p.bands, p.kqm, iq, ik, sqv), None

    me = peps.MatrixElements2Band(calc_minm, w.npb)
    eps, e1, e2, head = me.calc_eps(p.qs[0], None, None, None, None, p.kqm, p.bands, None, None, None, None, None,
                                    p.fr, kcw, None, None, None, None)
    ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb)
    assert e1 is None and eps.shape == (w.npb, w.npb, kcw.shape[-1])
    assert _rel(eps, ref[0]) < TOL


def test_chi0_input_paths_agree():
    """Per-k callable, device-resident tensor and pinned host tensor (streamed
    in double-buffered k-chunks on a side stream) give the same χ0."""
    w, p, kcw, minm = _problem()
    nb1, nb2, nkp, nom = kcw.shape
    P = nb1 * nb2
    kd = peps._kcw_device(kcw)
    a, _ = peps.chi0_accumulate(kd, lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom, k_chunk=7)
    host = torch.from_numpy(np.stack([m.reshape(P, w.npb) for m in minm])).pin_memory()
    b, _ = peps.chi0_accumulate(kd, host.cuda(), nkp, w.npb, nb1, nb2, nom)
    c, _ = peps.chi0_accumulate(kd, host, nkp, w.npb, nb1, nb2, nom, k_chunk=5)
    torch.cuda.synchronize()
    a, b, c = (x.cpu().numpy() for x in (a, b, c))
    assert _rel(b, a) < 1e-13 and _rel(c, a) < 1e-13


def test_weights_from_pinned_tensors_match_numpy_inputs():
    from pygw_gb300 import polarization as pol
    w, p, kcw, minm = _problem()
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    enk_h = torch.from_numpy(np.ascontiguousarray(b.enk().T)).pin_memory()
    tetc_h = torch.from_numpy(np.ascontiguousarray(p.kqm.tetc.T.astype(np.int32))).pin_memory()
    kq_h = torch.from_numpy(np.ascontiguousarray(p.kqm.kqid[:, iq].astype(np.int32))).pin_memory()
    om_h = torch.from_numpy(p.fr.omega.copy()).pin_memory()
    r = pol.weights_device(enk_h, b.EF, kq_h, 0, nomx, numin, om_h, tetc_h)
    torch.cuda.synchronize()
    assert np.array_equal(r.numpy(), kcw)
