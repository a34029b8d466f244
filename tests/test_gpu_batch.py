"""The batched driver (uneven N per q, ragged per-k windows, one CUDA graph):
each q against the FP64 oracle on the same matrix elements, and the graph
replay against the eager enqueue."""
import numpy as np
import pytest
import torch

from oracle import eps as oe
from oracle import weights as ow
from pygw_gb300 import _lib
from pygw_gb300 import batch as pb
from pygw_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _matrix_elements(bt, i, nb1, nb2):
    """The device generator's values for q i on the full window, as the oracle's per-k arrays."""
    lib = _lib.load()
    t = bt.tasks[i]
    rows = bt.nkp * nb1 * nb2
    out = torch.empty((rows, t.npb), dtype=torch.complex128, device="cuda")
    rc = lib.pg_synth_minm(bt.nkp, 0, t.iq, bt.enk_d.data_ptr(), bt.nbnd, bt.kqid_d[t.iq].data_ptr(), bt.ncg,
                           bt.numin, nb1, nb2, None, None, 0, bt.sqv_d[i].data_ptr(), t.npb, bt.seed,
                           out.data_ptr(), None)
    assert rc == 0
    m = out.cpu().numpy().reshape(bt.nkp, nb1, nb2, t.npb)
    for ik in range(bt.nkp):
        m[ik, :, bt.knb2[i][ik]:, :] = 0.0          # outside this k's window
    return m


def test_batch_uneven_q_matches_oracle_and_graph_equals_eager():
    w = syn.scaled(syn.WORKLOADS["C4"], div=3, nbands=40, nocc=6, nom=4, nq=3, npb_range=(70, 200))
    prob = syn.Problem(w)
    b = prob.bands
    tasks = pb.c4_tasks(prob, cut_lo=10, cut_hi=30)
    bt = pb.batch_for(prob, tasks, tuner=pb.Tuner(probe_nom=2))
    bt.run(graph=False)
    eager = [r.clone() for r in bt.results]
    bt.run(graph=True)
    assert bt.status() == 0
    nomx, numin = b.nomax_numin
    for i, t in enumerate(tasks):
        assert torch.equal(eager[i], bt.results[i])
        kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, prob.kqm.kqid[:, t.iq], 0, nomx, numin, prob.fr.omega,
                                   prob.kqm.tetc)
        m = _matrix_elements(bt, i, b.nb1, b.nb2)
        ref = oe.calc_eps(kcw, lambda ik: m[ik], t.npb)[0]
        got = bt.results[i].cpu().numpy().transpose(2, 1, 0)
        n = t.npb
        rel = max(np.max(np.abs(got[..., o] - ref[..., o])) / np.max(np.abs(ref[..., o] + np.eye(n)))
                  for o in range(w.nom))
        assert rel < 1e-9, (i, t.npb, rel)


def test_batch_q0_wings_and_head_match_oracle():
    """The large workload's q list at a small size: q = Γ with wings and the
    head formed from its weights on the device, against the FP64 oracle."""
    w = syn.scaled(syn.WORKLOADS["C5"], div=3, nbands=36, nocc=6, npb=96, nom=5, nq=2)
    prob = syn.Problem(w)
    b = prob.bands
    tasks = pb.c5_tasks(prob)
    assert tasks[0].iq == 0 and tasks[0].pm is not None
    # tuned: the tuner's probes of the q = Γ task run before the results exist
    bt = pb.batch_for(prob, tasks, tuner=pb.Tuner(probe_nom=2))
    bt.run(graph=True)
    assert bt.status() == 0
    nomx, numin = b.nomax_numin
    t = tasks[0]
    kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, prob.kqm.kqid[:, 0], 0, nomx, numin, prob.fr.omega, prob.kqm.tetc)
    m = _matrix_elements(bt, 0, b.nb1, b.nb2)
    pms = [t.pm[ik] for ik in range(bt.nkp)]
    head = syn.head_from_weights(kcw, pms)
    ref = oe.calc_eps(kcw, lambda ik: m[ik], t.npb, pm_k=lambda ik: pms[ik], head=head)
    got = bt.results[0].cpu().numpy().transpose(2, 1, 0)
    q = bt.q0[0]
    for a, e in ((got, ref[0]), (q["w1"].cpu().numpy().T, ref[1]), (q["w2"].cpu().numpy().T, ref[2]),
                 (q["head"].cpu().numpy(), ref[3])):
        assert np.max(np.abs(a - e)) <= 1e-9 * max(1.0, np.max(np.abs(e)))
