"""Replica split of the q points over ranks (the reference's mpiSplitArray)
and the host side of a multi-rank run on CPU with the gloo backend: each rank
runs its own q points, the per-q results are summed on rank 0 as the
reference reduces its self-energies, and the step time is the maximum over
ranks."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pygw_gb300 import replicas


@pytest.mark.parametrize("size,n", [(1, 5), (2, 5), (3, 9), (4, 10), (8, 3), (5, 2), (2, 1)])
def test_split_covers_every_point_once(size, n):
    taken = []
    for r in range(size):
        s, e = replicas.split_range(r, size, n)
        assert 0 <= s <= e <= n
        taken.extend(range(s, e))
    if size <= n:
        assert sorted(taken) == list(range(n))
    else:
        assert len(set(taken)) == len(taken) and set(taken) <= set(range(n))
    s, e, counts, displ = replicas.split(0, size, n)
    assert counts.sum() == len(taken) and len(displ) == size


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, size, port, nq, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    from oracle import weights as ow
    from pygw_gb300 import synthetic as syn
    w = syn.scaled(syn.WORKLOADS["C1"], div=2, nom=3, nq=nq)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    acc = torch.zeros(nq, dtype=torch.float64)
    for iq_pos in range(*replicas.split_range(rank, size, len(p.qs))):
        iq = p.qs[iq_pos]
        kcw = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)
        acc[iq_pos] = float(np.sum(kcw))
    dist.reduce(acc, dst=0, op=dist.ReduceOp.SUM)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((acc.numpy().tolist(), float(t.item())))
    dist.destroy_process_group()


def test_two_ranks_split_and_reduce_like_one():
    nq = 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, nq, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    sums, tmax = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=300)
        assert pr.exitcode == 0
    from oracle import weights as ow
    from pygw_gb300 import synthetic as syn
    w = syn.scaled(syn.WORKLOADS["C1"], div=2, nom=3, nq=nq)
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    ref = [float(np.sum(ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega,
                                             p.kqm.tetc))) for iq in p.qs]
    assert np.allclose(sums, ref, rtol=0, atol=0)
    assert tmax == 2.0
