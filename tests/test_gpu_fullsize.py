"""The split-precision path against the FP64 path at the full C3 matrix size.

C3 has N_PB = 1200 (2,560 padded rows in the digit GEMM: ten 256-column
blocks, 55 cluster blocks), 48 frequencies and 23 × 192 band pairs per k.
The FP64 contraction of all 216 k-points takes minutes, so both paths
contract the same two-point slice of the 6³ k-mesh (K = 8,832) with the
weights of the full mesh, then build and invert ε.  The tolerance of the
small cases (ε⁻¹ within 1e-9, max |Δ| over max |ε⁻¹| per frequency) must hold
at the full dimension, and the inverse must be Hermitian as ε is.  (The FP64
path itself is checked against the numpy oracle at smaller sizes.)
"""
import pytest
import torch

from pygw_gb300 import eps as peps
from pygw_gb300 import polarization as pol
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def test_c3_full_dimension_mixed_matches_fp64_on_a_k_slice():
    w = syn.WORKLOADS["C3"]
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    r = pol.weights_device(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    torch.cuda.synchronize()
    assert r.status == 0
    nom, nkp, nb2, nb1 = r.kcw.shape
    assert (nom, nkp, nb1, nb2) == (w.nom, p.kqm.nkp, b.nb1, b.nb2)
    nk = 2
    kcw = r.kcw[:, :nk].contiguous()
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    m = torch.stack([torch.from_numpy(syn.minm_k(w, b, p.kqm, iq, ik, sqv).reshape(nb1 * nb2, w.npb))
                     for ik in range(nk)]).cuda()
    ref = peps.chi0_eps(kcw, m, nk, w.npb, nb1, nb2, nom, precision="fp64")
    got = peps.chi0_eps(kcw, m, nk, w.npb, nb1, nb2, nom, precision="mixed")
    torch.cuda.synchronize()
    assert int(got.chi0_status.item()) == 0
    eye = torch.eye(w.npb, dtype=torch.complex128, device="cuda")
    einv_ref = ref.eps + eye
    einv = got.eps + eye
    rel = ((einv - einv_ref).abs().amax(dim=(1, 2)) / einv_ref.abs().amax(dim=(1, 2))).max().item()
    herm = ((einv - einv.conj().transpose(1, 2)).abs().amax(dim=(1, 2)) / einv.abs().amax(dim=(1, 2))).max().item()
    print(f"C3 dimension, {nk} k-points: eps^-1 max rel {rel:.2e}, hermiticity {herm:.2e}")
    assert rel < 1e-9, rel
    assert herm < 1e-9, herm
