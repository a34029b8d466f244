"""Device-side synthetic matrix elements (pg_synth_minm): distribution, and the
same values whichever k-chunk or window layout they are drawn in."""
import numpy as np
import pytest
import torch

from pygw_gb300 import _lib
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _setup():
    w = syn.scaled(syn.WORKLOADS["C1"], div=3, npb=200, nom=2)
    p = syn.Problem(w)
    b = p.bands
    iq = p.qs[0]
    enk = torch.from_numpy(np.ascontiguousarray(b.enk().T)).cuda()          # [nkp][nbnd]
    kq = torch.from_numpy(np.ascontiguousarray(p.kqm.kqid[:, iq].astype(np.int32))).cuda()
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    return w, p, b, iq, enk, kq, sqv


def _gen(lib, nk, k0, iq, enk, nbnd, kq, b, sqv_d, N, kstart=None, knb2=None, nrows=0):
    rows = nrows if kstart is not None else nk * b.nb1 * b.nb2
    out = torch.empty((rows, N), dtype=torch.complex128, device="cuda")
    rc = lib.pg_synth_minm(nk, k0, iq, enk.data_ptr(), nbnd, kq.data_ptr(), b.ncg_p, b.nomax_numin[1], b.nb1, b.nb2,
                           kstart.data_ptr() if kstart is not None else None,
                           knb2.data_ptr() if knb2 is not None else None, nrows, sqv_d.data_ptr(), N, 1234,
                           out.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_distribution_and_chunk_independence():
    w, p, b, iq, enk, kq, sqv = _setup()
    lib = _lib.load()
    nkp, nbnd, N = p.kqm.nkp, enk.shape[1], w.npb
    sqv_d = torch.from_numpy(sqv).cuda()
    full = _gen(lib, nkp, 0, iq, enk, nbnd, kq, b, sqv_d, N)
    # expected scale per (k, p, I): 1/(1+|ΔE|)·√v_I
    e = b.enk()
    numin = b.nomax_numin[1]
    scale = []
    for ik in range(nkp):
        jk = int(p.kqm.kqid[ik, iq])
        d = np.abs(e[:b.nb1, ik][:, None] - e[numin:numin + b.nb2, jk][None, :]).reshape(-1)
        scale.append(1.0 / (1.0 + d))
    scale = np.concatenate(scale)[:, None] * sqv[None, :]
    z = full / scale                              # ~ CN(0,1): E|z|² = 1, E z = 0
    n = z.size
    assert abs(np.mean(np.abs(z) ** 2) - 1.0) < 6.0 / np.sqrt(n)
    assert abs(np.mean(z.real)) < 6.0 / np.sqrt(n) and abs(np.mean(z.imag)) < 6.0 / np.sqrt(n)
    assert abs(np.mean(z.real ** 2) - 0.5) < 6.0 / np.sqrt(n)
    # a chunk drawn alone equals the same rows of the full draw
    P = b.nb1 * b.nb2
    part = _gen(lib, 4, 5, iq, enk, nbnd, kq, b, sqv_d, N)
    assert np.array_equal(part, full[5 * P:9 * P])


def test_ragged_windows_select_the_same_values():
    w, p, b, iq, enk, kq, sqv = _setup()
    lib = _lib.load()
    nkp, nbnd, N = p.kqm.nkp, enk.shape[1], w.npb
    sqv_d = torch.from_numpy(sqv).cuda()
    full = _gen(lib, nkp, 0, iq, enk, nbnd, kq, b, sqv_d, N).reshape(nkp, b.nb1, b.nb2, N)
    rng = np.random.default_rng(3)
    knb2 = rng.integers(1, b.nb2 + 1, size=nkp).astype(np.int32)
    kstart = np.concatenate([[0], np.cumsum(b.nb1 * knb2)]).astype(np.int32)
    rag = _gen(lib, nkp, 0, iq, enk, nbnd, kq, b, sqv_d, N, torch.from_numpy(kstart).cuda(),
               torch.from_numpy(knb2).cuda(), int(kstart[-1]))
    for ik in range(nkp):
        blk = rag[kstart[ik]:kstart[ik + 1]].reshape(b.nb1, knb2[ik], N)
        assert np.array_equal(blk, full[ik, :, :knb2[ik], :])     # keyed by (q, k, n, m, I)
    assert rag.shape[0] == int(kstart[-1])
