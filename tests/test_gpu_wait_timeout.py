"""Expiry of the digit GEMM's bounded pipeline waits (GPU, through the C-ABI).

Every wait inside k_ozaki_gemm (a TMA stage landing, the MMAs releasing a
stage, a chunk of the accumulator becoming readable) gives up after a limit
of the GPU's global timer.  The reference has no such failure mode: where its
Fortran meets an impossible state it stops the process
(for_tetrahedra2.f90:1777-1781); here a launch reports PG_ERR_TIMEOUT in its
status word and returns, leaving the context usable.

The test makes the waits expire on purpose by setting a limit of 200 ns
(``pg_set_wait_limit_ns``) — far below the microseconds one chunk of MMAs
takes — and checks that
  * the launch returns and its status word carries PG_ERR_TIMEOUT,
  * the unfinished output is marked (non-finite values), not silently wrong,
  * with the default limit restored, the next launches are clean and give
    bit-identical results to a launch made before the expiry.
No GPU fault, trap or hang is involved: the expiry is an ordinary branch of
the kernel that drains its own in-flight copies and MMAs before it exits.
"""
import pytest
import torch

from oracle import weights as ow
from pygw_gb300 import _lib
from pygw_gb300 import eps as peps
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
PG_ERR_TIMEOUT = 1 << 7


def _case():
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=100, nom=3)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    minm = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in range(p.kqm.nkp)]
    return w, kcw, minm


def _run(w, kcw, minm):
    nb1, nb2, nkp, nom = kcw.shape
    eps, status, _ = peps.chi0_mixed(peps._kcw_device(kcw), lambda ik: minm[ik], nkp, w.npb, nb1, nb2, nom,
                                     omega_batch=2, kb_split=100)
    torch.cuda.synchronize()
    return eps, int(status.item())


def test_expired_waits_report_timeout_and_leave_the_context_usable():
    lib = _lib.load()
    w, kcw, minm = _case()
    assert lib.pg_wait_limit_ns() == 5_000_000_000
    eps0, st0 = _run(w, kcw, minm)
    assert st0 == 0 and torch.isfinite(torch.view_as_real(eps0)).all()
    lib.pg_set_wait_limit_ns(200)
    try:
        assert lib.pg_wait_limit_ns() == 200
        eps1, st1 = _run(w, kcw, minm)
    finally:
        lib.pg_set_wait_limit_ns(0)
    assert lib.pg_wait_limit_ns() == 5_000_000_000
    assert st1 & PG_ERR_TIMEOUT
    assert not torch.isfinite(torch.view_as_real(eps1)).all()
    for _ in range(2):
        eps2, st2 = _run(w, kcw, minm)
        assert st2 == 0
        assert torch.equal(eps2, eps0)
