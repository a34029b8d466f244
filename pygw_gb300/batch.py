"""Many q points of uneven shape through the GPU path, captured in one CUDA graph.

The reference loops over q in ``G0W0.Compute`` (pygw.py:3659-3711): for each q
``Polarization_weights`` (pygw.py:3416) then ``calc_eps`` (pygw.py:3039), with
the q list split over MPI ranks.  This module runs a list of q points back to
back on one GPU with everything enqueued on one stream and no host
synchronisation, so the whole batch is captured once as a CUDA graph and
replayed (``run(graph=True)``):

* per q: tetrahedron weights (``pg_bz_calcqdepw_par2``), then for each
  k-chunk the matrix elements (``pg_synth_minm``, drawn on the device from the
  workload seed — a caller with its own matrix elements uses
  ``eps.chi0_accumulate`` per q) and the
  split-precision contraction with ragged per-k band windows
  (``pg_chi0_mixed_accumulate``), then the mixed-precision ε⁻¹
  (``pg_eps_inverse_mixed``);
* q points have their own product-basis size N_q and their own per-k
  unoccupied-band windows; buffers and workspaces are allocated once for the
  largest q and reused;
* ``Tuner`` picks the k-chunk and the frequency batch of the contraction per
  shape class (N_q rounded up to 256 and the window total) by timing
  candidates on a few frequencies, before capture.

``Batch.results[i]`` is ε⁻¹ − 1 of q i as a CUDA tensor ``[nom][N][N]``
(Fortran ``(N, N, nom)`` storage, as ``calc_eps`` returns it).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from . import eps as peps
from .device import free_device_bytes, ptr, require_cuda, stream_handle

FSPIN = 2.0


@dataclass
class QTask:
    """One q point: its kqid column index, N_q, √v_I and per-k windows."""
    iq: int
    npb: int
    sqv: np.ndarray                      # √v_I, length npb
    knb2: np.ndarray | None = None       # per-k unoccupied bands in the window (None: all nb2)
    pm: np.ndarray | None = None         # q → 0: wing vectors [nkp][nb1·nb2] (full window only)
    head: np.ndarray | None = None       # q → 0: head [nom] (FP64 complex); None with pm: the synthetic
    #                                      head −2 Σ_k Σ_p |pm|²·w from this q's weights, formed on the device


@dataclass
class TuneChoice:
    k_chunk: int
    omega_batch: int
    ms_per_omega: float = 0.0


class Tuner:
    """Chooses (k_chunk, omega_batch) of the split-precision contraction per
    shape class by timing each candidate on ``probe_nom`` frequencies.  Results
    are kept in memory and, with ``path``, in a JSON file keyed by the class."""

    def __init__(self, path: str | None = None, probe_nom: int = 4):
        self.path = path
        self.probe_nom = probe_nom
        self.table: dict[str, dict] = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.table = json.load(f)

    @staticmethod
    def key(npb, nb1, nb2, nkp, ktot, nom):
        return f"N{-(-npb // 256) * 256}_nb{nb1}x{nb2}_k{nkp}_K{-(-ktot // 65536)}_w{nom}"

    def save(self):
        if self.path:
            with open(self.path, "w") as f:
                json.dump(self.table, f, indent=1, sort_keys=True)

    def choose(self, key, candidates, timer):
        if key in self.table:
            c = self.table[key]
            return TuneChoice(c["k_chunk"], c["omega_batch"], c.get("ms_per_omega", 0.0))
        best = None
        for kc, wb in candidates:
            ms = timer(kc, wb)
            if best is None or ms < best.ms_per_omega:
                best = TuneChoice(kc, wb, ms)
        self.table[key] = {"k_chunk": best.k_chunk, "omega_batch": best.omega_batch,
                           "ms_per_omega": best.ms_per_omega,
                           "candidates": [[kc, wb] for kc, wb in candidates]}
        self.save()
        return best


class Batch:
    """Static inputs of one mesh/band structure and a list of ``QTask``s."""

    def __init__(self, enk, ef, kqid, tetc, ncg, nomx, numin, omega, tasks, seed=0, k_chunk=None, omega_batch=None,
                 refine_iters=None, tuner: Tuner | None = None, mem_fraction=0.6):
        require_cuda()
        self.lib = _lib.load()
        self.tasks = list(tasks)
        enk = np.asarray(enk, dtype=np.float64)
        self.nbnd, self.nkp = enk.shape
        self.ef, self.ncg, self.nomx, self.numin = float(ef), int(ncg), int(nomx), int(numin)
        self.nb1 = ncg + nomx + 1
        self.nb2 = self.nbnd - ncg - numin
        self.omega = np.asarray(omega, dtype=np.float64)
        self.nom = len(self.omega)
        self.ntet = np.asarray(tetc).shape[1]
        self.seed = int(seed)
        self.refine_iters = refine_iters
        # static device inputs (weights' C-ABI layouts)
        self.enk_d = torch.from_numpy(np.ascontiguousarray(enk.T)).cuda()                       # [nkp][nbnd]
        self.tetc_d = torch.from_numpy(np.ascontiguousarray(np.asarray(tetc).T.astype(np.int32))).cuda()
        kq = np.asarray(kqid)
        self.kqid_d = {t.iq: torch.from_numpy(np.ascontiguousarray(kq[:, t.iq].astype(np.int32))).cuda()
                       for t in self.tasks}
        self.om_d = torch.from_numpy(self.omega.copy()).cuda()
        self.sqv_d = [torch.from_numpy(np.asarray(t.sqv, dtype=np.float64)).cuda() for t in self.tasks]
        self.kcw = torch.empty((self.nom, self.nkp, self.nb2, self.nb1), dtype=torch.float64, device="cuda")
        # weight scratch: all frequencies at once unless that exceeds a quarter of the free memory
        free0 = free_device_bytes()
        self.nom_chunk = self.nom
        while self.nom_chunk > 1 and self.lib.pg_bz_calcqdepw_par2_workspace(
                self.nbnd, self.nkp, ncg, nomx, numin, self.nom, self.ntet, self.nom_chunk) > free0 // 4:
            self.nom_chunk = (self.nom_chunk + 1) // 2
        wbytes = self.lib.pg_bz_calcqdepw_par2_workspace(self.nbnd, self.nkp, ncg, nomx, numin, self.nom, self.ntet,
                                                         self.nom_chunk)
        self.wwork = torch.empty(wbytes, dtype=torch.uint8, device="cuda")
        # q → 0: wings and head (uniform windows)
        self.q0 = {}
        for i, t in enumerate(self.tasks):
            if t.pm is None:
                continue
            if t.knb2 is not None and np.any(np.asarray(t.knb2) < self.nb2):
                raise ValueError("q → 0 wings need the full band window")
            self.q0[i] = {"pm": torch.from_numpy(np.ascontiguousarray(t.pm, dtype=np.complex128)).cuda(),
                          "head0": (None if t.head is None else
                                    torch.from_numpy(np.asarray(t.head, dtype=np.complex128).copy()).cuda()),
                          "pm2": torch.from_numpy(np.abs(np.asarray(t.pm)) ** 2).cuda(),
                          "head": torch.empty(self.nom, dtype=torch.complex128, device="cuda"),
                          "hre": torch.empty(self.nom, dtype=torch.float64, device="cuda"),
                          "w1": torch.empty((self.nom, t.npb), dtype=torch.complex128, device="cuda"),
                          "w2": torch.empty((self.nom, t.npb), dtype=torch.complex128, device="cuda")}
        self.wstatus = torch.zeros(len(self.tasks), dtype=torch.int32, device="cuda")
        # per-q window bookkeeping
        self.knb2 = [np.full(self.nkp, self.nb2, dtype=np.int32) if t.knb2 is None
                     else np.minimum(np.asarray(t.knb2, dtype=np.int32), self.nb2) for t in self.tasks]
        self.ktot = [int(self.nb1 * kn.sum()) for kn in self.knb2]
        # tuning (before any buffer sized by the choice is allocated)
        free = free_device_bytes()
        results_bytes = sum(16 * self.nom * t.npb * t.npb for t in self.tasks)
        eps_ws = max(self.lib.pg_eps_inverse_mixed_workspace(t.npb, self.nom, 0) for t in self.tasks)
        self.budget = max(1 << 28, int(mem_fraction * free) - results_bytes - eps_ws)
        self.choice = []
        for i, t in enumerate(self.tasks):
            if k_chunk is not None or omega_batch is not None or tuner is None:
                kc = k_chunk or self._default_k_chunk(t.npb, self.knb2[i])
                wb = omega_batch or self._fit_omega_batch(t.npb, kc)
                self.choice.append(TuneChoice(kc, wb))
            else:
                key = Tuner.key(t.npb, self.nb1, self.nb2, self.nkp, self.ktot[i], self.nom)
                self.choice.append(tuner.choose(key, self._candidates(t.npb, self.knb2[i]),
                                                lambda kc, wb, i=i: self._probe(i, kc, wb, tuner.probe_nom)))
        # buffers for the largest q
        self._alloc()
        self.graph = None

    # ---------------------------------------------------------------- sizing
    def _rows(self, i, k0, kc):
        return int(self.nb1 * self.knb2[i][k0:k0 + kc].sum())

    def _default_k_chunk(self, npb, knb2):
        per_k = self.nb1 * int(knb2.max()) * npb * 16
        return int(max(1, min(self.nkp, (self.budget // 4) // max(1, per_k))))

    def _fit_omega_batch(self, npb, kc):
        wb = 1
        while wb < self.nom and self.lib.pg_chi0_mixed_workspace(self.nb1, self.nb2, kc, npb, 2 * wb, 0) + \
                self.nb1 * self.nb2 * kc * npb * 16 <= self.budget:
            wb *= 2
        return min(wb, self.nom)

    def _candidates(self, npb, knb2):
        kmax = self._default_k_chunk(npb, knb2)
        kcs = sorted({kmax, max(1, kmax // 2)}, reverse=True)
        out = []
        for kc in kcs:
            wfit = self._fit_omega_batch(npb, kc)
            for wb in sorted({wfit, max(1, wfit // 2), 1}, reverse=True):
                out.append((kc, wb))
        return out

    def _alloc(self):
        rows = max(max(self._rows(i, k0, c.k_chunk) for k0 in range(0, self.nkp, c.k_chunk))
                   for i, c in enumerate(self.choice))
        nmax = max(t.npb for t in self.tasks)
        self.m_buf = torch.empty((rows, nmax), dtype=torch.complex128, device="cuda")
        cbytes = max(self.lib.pg_chi0_mixed_workspace(self.nb1, self.nb2, c.k_chunk, t.npb, c.omega_batch, 0)
                     for t, c in zip(self.tasks, self.choice))
        self.cwork = torch.empty(cbytes, dtype=torch.uint8, device="cuda")
        self.cstatus = torch.zeros(len(self.tasks), dtype=torch.int32, device="cuda")
        self.estatus = torch.zeros(len(self.tasks), dtype=torch.int32, device="cuda")
        ebytes = max(self.lib.pg_eps_inverse_mixed_workspace(t.npb, self.nom, 0) for t in self.tasks)
        self.ework = torch.empty(ebytes, dtype=torch.uint8, device="cuda")
        self.results = [torch.empty((self.nom, t.npb, t.npb), dtype=torch.complex128, device="cuda")
                        for t in self.tasks]
        # per-(q, chunk) ragged offsets on the device
        self.kstart_d = []
        for i, c in enumerate(self.choice):
            per = []
            for k0 in range(0, self.nkp, c.k_chunk):
                kc = min(c.k_chunk, self.nkp - k0)
                kn = self.knb2[i][k0:k0 + kc]
                ks = np.concatenate([[0], np.cumsum(self.nb1 * kn)]).astype(np.int32)
                per.append((k0, kc, int(ks[-1]), torch.from_numpy(ks).cuda(),
                            torch.from_numpy(np.ascontiguousarray(kn)).cuda()))
            self.kstart_d.append(per)

    # ------------------------------------------------------------- enqueue
    def _check(self, rc, what):
        _lib.check(rc, what)

    def _weights(self, i, sh):
        t = self.tasks[i]
        rc = self.lib.pg_bz_calcqdepw_par2(ptr(self.enk_d), self.nbnd, self.nkp, self.ef, ptr(self.kqid_d[t.iq]),
                                           self.ncg, self.nomx, self.numin, ptr(self.om_d), self.nom,
                                           ptr(self.tetc_d), self.ntet, ptr(self.kcw), ptr(self.wwork),
                                           self.wwork.numel(), self.nom_chunk, ptr(self.wstatus[i:i + 1]), None, sh)
        self._check(rc, "pg_bz_calcqdepw_par2")

    def _chi0(self, i, sh, nom, chunks, wb, eps):
        t = self.tasks[i]
        N = t.npb
        for c, (k0, kc, rows, ks, kn) in enumerate(chunks):
            mv = self.m_buf.view(-1)[:rows * N]
            rc = self.lib.pg_synth_minm(kc, k0, t.iq, ptr(self.enk_d), self.nbnd, ptr(self.kqid_d[t.iq]), self.ncg,
                                        self.numin, self.nb1, self.nb2, ptr(ks), ptr(kn), rows, ptr(self.sqv_d[i]),
                                        N, self.seed, ptr(mv), sh)
            self._check(rc, "pg_synth_minm")
            rc = self.lib.pg_chi0_mixed_accumulate(ptr(mv), kc, k0, ptr(ks), ptr(kn), rows, ptr(self.kcw), self.nb1,
                                                   self.nb2, self.nkp, nom, N, -FSPIN, ptr(eps), 1 if c > 0 else 0,
                                                   ptr(self.cwork), self.cwork.numel(), wb, 0,
                                                   ptr(self.cstatus[i:i + 1]), sh, None)
            self._check(rc, "pg_chi0_mixed_accumulate")
            # the wings belong to the batch's own result (not to a tuning probe,
            # which runs before the results exist)
            if i in self.q0 and eps is getattr(self, "results", [None] * (i + 1))[i]:
                q = self.q0[i]
                rc = self.lib.pg_wings_f64(ptr(mv), kc, k0, ptr(self.kcw), self.nb1, self.nb2, self.nkp, nom, N,
                                           -FSPIN, ptr(q["pm"][k0:k0 + kc]), ptr(q["w1"]), sh)
                self._check(rc, "pg_wings_f64")

    def enqueue(self):
        """All launches of the batch on the current stream (no host synchronisation)."""
        sh = stream_handle(None)
        iters = peps.REFINE_ITERS if self.refine_iters is None else self.refine_iters
        for i, t in enumerate(self.tasks):
            self._weights(i, sh)
            c = self.choice[i]
            eps = self.results[i]
            q = self.q0.get(i)
            if q is not None:
                q["w1"].zero_()
                if q["head0"] is not None:
                    q["head"].copy_(q["head0"])
                else:
                    # synthetic head from the weights: kcw [ω][k][m][n] → pair n·nb2 + m as pm
                    w = self.kcw.permute(0, 1, 3, 2).reshape(self.nom, self.nkp, -1)
                    torch.mul(torch.einsum("wkp,kp->w", w, q["pm2"]), -2.0, out=q["hre"])
                    q["head"].copy_(q["hre"])
            self._chi0(i, sh, self.nom, self.kstart_d[i], c.omega_batch, eps)
            if q is not None:
                torch.conj_physical(q["w1"], out=q["w2"])
            rc = self.lib.pg_eps_inverse_mixed(ptr(eps), t.npb, self.nom, ptr(q["w1"]) if q else None,
                                               ptr(q["w2"]) if q else None, ptr(q["head"]) if q else None,
                                               ptr(self.ework), self.ework.numel(), 0, int(iters),
                                               ptr(self.estatus[i:i + 1]), sh)
            self._check(rc, "pg_eps_inverse_mixed")

    def capture(self):
        """Record the batch as one CUDA graph (after one uncaptured run)."""
        self.enqueue()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        l0 = self.lib.pg_launch_count()
        with torch.cuda.graph(g):
            self.enqueue()
        torch.cuda.synchronize()
        self.graph_launches = int(self.lib.pg_launch_count() - l0)      # kernels per replay
        self.graph = g
        return g

    def run(self, graph=True):
        if graph:
            if self.graph is None:
                self.capture()
            self.graph.replay()
        else:
            self.enqueue()

    def status(self):
        """OR of every kernel status word of the last run (0 = clean)."""
        torch.cuda.synchronize()
        s = 0
        for t in (self.wstatus, self.cstatus, self.estatus):
            for v in t.cpu().tolist():
                s |= int(v)
        return s

    # -------------------------------------------------------------- tuning
    def _probe(self, i, kc, wb, probe_nom):
        """ms per frequency of the contraction of q i with (k_chunk, omega_batch)."""
        t = self.tasks[i]
        nom = min(probe_nom, self.nom)
        wb = min(wb, nom)
        chunks = []
        for k0 in range(0, self.nkp, kc):
            kcc = min(kc, self.nkp - k0)
            kn = self.knb2[i][k0:k0 + kcc]
            ks = np.concatenate([[0], np.cumsum(self.nb1 * kn)]).astype(np.int32)
            chunks.append((k0, kcc, int(ks[-1]), torch.from_numpy(ks).cuda(),
                           torch.from_numpy(np.ascontiguousarray(kn)).cuda()))
        rows = max(c[2] for c in chunks)
        saved = getattr(self, "m_buf", None), getattr(self, "cwork", None), getattr(self, "cstatus", None)
        self.m_buf = torch.empty((rows, t.npb), dtype=torch.complex128, device="cuda")
        self.cwork = torch.empty(self.lib.pg_chi0_mixed_workspace(self.nb1, self.nb2, kc, t.npb, wb, 0),
                                 dtype=torch.uint8, device="cuda")
        self.cstatus = torch.zeros(len(self.tasks), dtype=torch.int32, device="cuda")
        eps = torch.empty((nom, t.npb, t.npb), dtype=torch.complex128, device="cuda")
        sh = stream_handle(None)
        self._weights(i, sh)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        self._chi0(i, sh, nom, chunks, wb, eps)                  # warm-up
        ev[0].record()
        self._chi0(i, sh, nom, chunks, wb, eps)
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / nom
        self.m_buf, self.cwork, self.cstatus = saved
        del eps
        torch.cuda.empty_cache()
        return ms


def c4_tasks(problem, seed=0, cut_lo=100, cut_hi=300):
    """The batched workload's q list: N_q seeded in the workload's range and
    per-k unoccupied-band cutoffs seeded uniform in [cut_lo, cut_hi] bands."""
    from . import synthetic as syn
    w = problem.w
    b = problem.bands
    numin = b.nomax_numin[1]
    rng = np.random.default_rng([w.seed, 13])
    cut = rng.integers(cut_lo, cut_hi + 1, size=problem.kqm.nkp)
    knb2 = np.clip(cut - b.ncg_p - numin, 1, b.nb2).astype(np.int32)
    tasks = []
    for pos, iq in enumerate(problem.qs):
        n = syn.npb_for_q(w, pos)
        tasks.append(QTask(iq=iq, npb=n, sqv=syn.coulomb_sqrt(w, iq, n), knb2=knb2))
    return tasks


def batch_for(problem, tasks, **kw):
    """A ``Batch`` over a ``synthetic.Problem``'s mesh and bands."""
    b = problem.bands
    nomx, numin = b.nomax_numin
    return Batch(b.enk(), b.EF, problem.kqm.kqid, problem.kqm.tetc, b.ncg_p, nomx, numin, problem.fr.omega, tasks,
                 seed=problem.w.seed, **kw)


def c5_tasks(problem):
    """The large workload's q list: full band windows, the first q is Γ (q → 0)
    with synthetic wing vectors and the head formed from its weights."""
    from . import synthetic as syn
    w = problem.w
    b = problem.bands
    tasks = []
    for iq in problem.qs:
        t = QTask(iq=iq, npb=w.npb, sqv=syn.coulomb_sqrt(w, iq, w.npb))
        if iq == 0:
            t.pm = np.stack([syn.pm_k(w, b, ik) for ik in range(problem.kqm.nkp)])
        tasks.append(t)
    return tasks
