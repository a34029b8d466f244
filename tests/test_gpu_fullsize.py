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


def _c3_device_problem():
    """C3 weights of the first q and its matrix elements for all 216 k-points,
    drawn on the device by the synthetic generator (18 GB)."""
    import numpy as np
    from pygw_gb300 import _lib
    from pygw_gb300.device import ptr
    w = syn.WORKLOADS["C3"]
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    r = pol.weights_device(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    nom, nkp, nb2, nb1 = r.kcw.shape
    enk = b.enk()
    enk_d = torch.from_numpy(np.ascontiguousarray(enk.T)).cuda()
    kq_d = torch.from_numpy(np.ascontiguousarray(p.kqm.kqid[:, iq].astype(np.int32))).cuda()
    sqv_d = torch.from_numpy(syn.coulomb_sqrt(w, iq, w.npb)).cuda()
    m = torch.empty((nkp, nb1 * nb2, w.npb), dtype=torch.complex128, device="cuda")
    lib = _lib.load()
    _lib.check(lib.pg_synth_minm(nkp, 0, iq, ptr(enk_d), enk.shape[0], ptr(kq_d), 0, numin, nb1, nb2, None, None, 0,
                                 ptr(sqv_d), w.npb, w.seed, ptr(m), None), "pg_synth_minm")
    torch.cuda.synchronize()
    return w, r, m, nkp, nb1, nb2, nom


def test_c3_full_k_mesh_mixed_matches_fp64_elementwise():
    """The benchmarked configuration itself: all 216 k-points, N_PB = 1200, the
    lowest, a middle and the highest of the 48 frequencies.  Both paths get
    the same weights and matrix elements; the split-precision ε⁻¹ must agree
    with the FP64 one to 1e-9 normwise (max |Δ| over max |ε⁻¹|), and its
    element-wise relative error over the entries above 1e-8 of the largest is
    reported (see pygw_gb300.accuracy)."""
    from pygw_gb300 import accuracy
    w, r, m, nkp, nb1, nb2, nom = _c3_device_problem()
    acc = accuracy.mixed_vs_fp64(r.kcw, m, nkp, w.npb, nb1, nb2, [0, nom // 2, nom - 1])
    print(f"C3, all {nkp} k-points, frequencies {acc['frequencies']}: normwise {acc['normwise']}, "
          f"element-wise {acc['elementwise']}, diagonal {acc['diagonal']}")
    assert acc["status"] == 0
    assert acc["max_normwise"] < 1e-9, acc


def test_c3_full_weights_bit_exact():
    """The weights of the benchmarked configuration (200 bands, 6³ k, all 48
    frequencies, the first q) against the oracle, bit for bit."""
    import numpy as np
    from oracle import weights as ow
    w = syn.WORKLOADS["C3"]
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    args = (b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    ref, st_ref, stats = ow.bz_calcqdepw_par2(*args, return_stats=True)
    r = pol.weights_device(*args)
    torch.cuda.synchronize()
    got = r.numpy()
    assert got.shape == ref.shape == (b.nb1, b.nb2, p.kqm.nkp, w.nom)
    assert r.status == st_ref and r.counters == stats
    assert np.array_equal(got, ref), np.abs(got - ref).max()
