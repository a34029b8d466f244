"""Split-precision χ0 on the tensor cores (sm_103a, through the C-ABI).

1. White box: the digits the GPU produced are read back from its workspace,
   every digit-group integer I_d = Σ_{s+t=d} Σ_K a_s b_t is recomputed
   exactly in numpy (float64 sums of small integers below 2^53), and the
   kernel's output tiles must match bit for bit — this checks the TMA
   layout, the MMA descriptors, the exactness of the FP32 tensor-core
   accumulation of integer products and the renormalisation between chunks.
2. The digits represent their values to the expected 2^-40 (row scale).
3. End to end: χ0 within 1e-10 of the FP64 oracle at each row/column scale
   (|Δχ0_IJ| ≤ tol·sqrt(|χ0_II χ0_JJ|)) and ε⁻¹ within 1e-9 (max relative).
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import eps as oe
from oracle import weights as ow
from pygw_gb300 import _lib
from pygw_gb300 import eps as peps
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
S = 5


def _problem(w):
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    minm = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in range(p.kqm.nkp)]
    return p, kcw, minm


def _bf16(u16):
    return (u16.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def test_digit_gemm_is_exact_white_box():
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=100, nom=3)
    p, kcw, minm = _problem(w)
    nb1, nb2, nkp, nom = kcw.shape
    P, N = nb1 * nb2, w.npb
    lib = _lib.load()
    kd = peps._kcw_device(kcw)
    wb, kb_split = 2, 100
    eps, status, work = peps.chi0_mixed(kd, lambda ik: minm[ik], nkp, N, nb1, nb2, nom, omega_batch=wb,
                                        kb_split=kb_split)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    offs = (ctypes.c_size_t * 9)()
    dims = (ctypes.c_longlong * 9)()
    assert lib.pg_chi0_mixed_layout(nb1, nb2, nkp, N, wb, kb_split, offs, dims) == 0
    K, K_pad, R, R_pad, nT, npair, nkb, nsplit, kbs = list(dims)
    assert nsplit >= 2 and nT == 2
    raw = work.cpu().numpy()

    def view(i, dtype, shape):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        return raw[offs[i]:offs[i] + n].view(dtype).reshape(shape)

    # the workspace holds the last preparation pass (wbp frequencies from op0)
    # and the last GEMM launch (frequencies from om0, B slot om0 − op0)
    wbp = -(-max(wb, lib.pg_chi0_prep_batch()) // wb) * wb
    om0 = (nom - 1) // wb * wb
    slot = om0 - om0 // wbp * wbp
    # digit arrays are K-block major: [plane][K-block][row][64]
    A = _bf16(view(0, np.uint16, (S, nkb, R_pad, 64)).transpose(0, 2, 1, 3).reshape(S, R_pad, K_pad))
    # (slots of the pass beyond nom were never written: only this one is read)
    B = _bf16(view(1, np.uint16, (wbp, S, nkb, R_pad, 64))[slot].transpose(0, 2, 1, 3).reshape(S, R_pad, K_pad))
    eA = view(5, np.int32, (R_pad,))
    fB = view(6, np.int32, (wbp, R_pad))[slot]
    out = view(7, np.float64, (nsplit, wb, npair, 128, 128))[:, 0]
    assert np.abs(A).max() <= 129 and np.abs(B).max() <= 129

    # (2) digits represent V and c·w·V
    M = np.concatenate([m.reshape(P, N) for m in minm])                    # [K, N]
    V = np.zeros((R_pad, K_pad))
    V[:N, :K] = M.real.T
    V[N:2 * N, :K] = M.imag.T
    scal = 2.0 ** -(8.0 * (np.arange(S) + 1))
    Vrec = np.einsum("srk,s->rk", A, scal) * 2.0 ** eA[:, None]
    assert np.all(np.abs(Vrec - V) <= 2.0 ** (eA[:, None] - 40.0))
    cw = -2.0 * np.array([kcw[:, :, ik, om0].ravel() for ik in range(nkp)]).ravel()
    cw = np.concatenate([cw, np.zeros(K_pad - K)])
    Brec = np.einsum("srk,s->rk", B, scal) * 2.0 ** fB[:, None]
    assert np.all(np.abs(Brec - Vrec * cw[None, :]) <= 2.0 ** (fB[:, None] - 38.0))

    # (1) exact group integers, combined in the kernel's order
    pair = 0
    for ti in range(nT):
        for tj in range(ti, nT):
            ra, rb = slice(128 * ti, 128 * ti + 128), slice(128 * tj, 128 * tj + 128)
            for sp in range(nsplit):
                ks = slice(sp * kbs * 64, min(K_pad, (sp + 1) * kbs * 64))
                acc = None
                for d in range(S):
                    I = sum(A[s, ra, ks] @ B[d - s, rb, ks].T for s in range(d + 1))
                    v = I * 2.0 ** (-8 * d)
                    acc = v if acc is None else acc + v
                got = out[sp, pair].T            # stored [col][row]
                assert np.array_equal(got, acc), (ti, tj, sp, np.abs(got - acc).max())
            pair += 1


def _row_scaled_err(a, ref):
    d = np.sqrt(np.abs(np.einsum("iiw->iw", ref)))
    return np.max(np.abs(a - ref) / (d[:, None, :] * d[None, :, :] + 1e-300))


@pytest.mark.parametrize("name,kw", [("C1", {}), ("C2", {"div": 4})])
def test_mixed_chi0_and_inverse_accuracy(name, kw):
    w = syn.scaled(syn.WORKLOADS[name], **kw) if kw else syn.WORKLOADS[name]
    p, kcw, minm = _problem(w)
    nb1, nb2, nkp, nom = kcw.shape
    ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb)
    chi0_ref = ref[4]
    chi0_ref = (chi0_ref + np.conj(chi0_ref.transpose(1, 0, 2))) / 2
    kd = peps._kcw_device(kcw)
    eps, status, _ = peps.chi0_mixed(kd, lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    chi0 = eps.cpu().numpy().transpose(2, 1, 0)
    e_chi0 = _row_scaled_err(chi0, chi0_ref)
    assert e_chi0 < 1e-10
    r = peps.chi0_eps(kcw, lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom, precision="mixed")
    einv = r.numpy()[0] + np.eye(w.npb)[:, :, None]
    einv_ref = ref[0] + np.eye(w.npb)[:, :, None]
    rel = max(np.max(np.abs(einv[..., o] - einv_ref[..., o])) / np.max(np.abs(einv_ref[..., o])) for o in range(nom))
    print(f"{name}: chi0 row-scaled {e_chi0:.2e}, eps^-1 max rel {rel:.2e}")
    assert rel < 1e-9, rel


def test_mixed_q0_wings_and_head():
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=96, nom=6)
    p, kcw, minm = _problem(w)
    nb1, nb2, nkp, nom = kcw.shape
    pms = [syn.pm_k(w, p.bands, ik) for ik in range(nkp)]
    head0 = syn.head_from_weights(kcw, pms)
    ref = oe.calc_eps(kcw, lambda ik: minm[ik], w.npb, pm_k=lambda ik: pms[ik], head=head0)
    r = peps.chi0_eps(kcw, lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom, pm_k=lambda ik: pms[ik], head=head0,
                      precision="mixed")
    eps, w1, w2, head = r.numpy()
    assert np.max(np.abs(head - ref[3])) / np.max(np.abs(ref[3])) < 1e-9
    assert np.max(np.abs(w1 - ref[1])) / np.max(np.abs(ref[1])) < 1e-9


def test_mixed_streamed_chunks_match_resident():
    """k-chunked split-precision χ0 (callable and pinned-host inputs, several
    chunks, q→0 wings) and the staged pinned-host path against the one-pass
    contraction over resident k."""
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=96, nom=4)
    p, kcw, minm = _problem(w)
    nb1, nb2, nkp, nom = kcw.shape
    P, N = nb1 * nb2, w.npb
    pms = [syn.pm_k(w, p.bands, ik) for ik in range(nkp)]
    kd = peps._kcw_device(kcw)
    eps_all, status, _ = peps.chi0_mixed(kd, lambda ik: minm[ik], nkp, N, nb1, nb2, nom)
    w1_all = peps.wings_f64(kd, lambda ik: minm[ik], nkp, N, nb1, nb2, nom, lambda ik: pms[ik])
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = eps_all.cpu().numpy().transpose(2, 1, 0)
    host = torch.from_numpy(np.stack([m.reshape(P, N) for m in minm])).pin_memory()
    # (host, None): pinned host input staged whole on a copy stream, one pass
    for src, kc in ((lambda ik: minm[ik], 3), (host, 4), (host, None)):
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        eps, w1 = peps.chi0_accumulate(kd, src, nkp, N, nb1, nb2, nom, pm_k=lambda ik: pms[ik], k_chunk=kc,
                                       precision="mixed", status=st)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        got = eps.cpu().numpy().transpose(2, 1, 0)
        assert _row_scaled_err(got, ref) < 1e-10      # each is within ~3e-11 of the FP64 oracle
        assert np.max(np.abs(w1.cpu().numpy() - w1_all.cpu().numpy())) <= 1e-12 * np.max(np.abs(w1_all.cpu().numpy()))


def test_mixed_ragged_windows_match_zero_padded():
    """Per-k unoccupied-band windows (ragged K = Σ_k nb1·knb2[k]) through the
    C-ABI against the uniform window with the excluded pairs' matrix elements
    set to zero (the same sum), and against the FP64 oracle."""
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=96, nom=3)
    p, kcw, minm = _problem(w)
    nb1, nb2, nkp, nom = kcw.shape
    N = w.npb
    rng = np.random.default_rng(12)
    knb2 = rng.integers(nb2 // 2, nb2 + 1, size=nkp).astype(np.int32)
    padded = []
    for ik in range(nkp):
        m = minm[ik].copy()
        m[:, knb2[ik]:, :] = 0.0
        padded.append(m)
    rag = np.concatenate([minm[ik][:, :knb2[ik], :].reshape(-1, N) for ik in range(nkp)])
    kstart = np.concatenate([[0], np.cumsum(nb1 * knb2)]).astype(np.int32)
    lib = _lib.load()
    kd = peps._kcw_device(kcw)
    wb = nom
    work = torch.empty(lib.pg_chi0_mixed_workspace(nb1, nb2, nkp, N, wb, 0), dtype=torch.uint8, device="cuda")
    eps = torch.empty((nom, N, N), dtype=torch.complex128, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    m_d, ks_d, kn_d = torch.from_numpy(rag).cuda(), torch.from_numpy(kstart).cuda(), torch.from_numpy(knb2).cuda()
    rc = lib.pg_chi0_mixed_accumulate(m_d.data_ptr(), nkp, 0, ks_d.data_ptr(), kn_d.data_ptr(), int(kstart[-1]),
                                      kd.data_ptr(), nb1, nb2, nkp, nom, N, -2.0, eps.data_ptr(), 0, work.data_ptr(),
                                      work.numel(), wb, 0, st.data_ptr(), None, None)
    assert rc == 0
    eps_u, st_u, _ = peps.chi0_mixed(kd, lambda ik: padded[ik], nkp, N, nb1, nb2, nom)
    torch.cuda.synchronize()
    assert int(st.item()) == 0 and int(st_u.item()) == 0
    got = eps.cpu().numpy().transpose(2, 1, 0)
    uni = eps_u.cpu().numpy().transpose(2, 1, 0)
    ref = oe.calc_eps(kcw, lambda ik: padded[ik], N)[4]
    ref = (ref + np.conj(ref.transpose(1, 0, 2))) / 2
    assert _row_scaled_err(got, ref) < 1e-10
    assert _row_scaled_err(got, uni) < 1e-10
