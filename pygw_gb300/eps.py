"""χ0 contraction and ε⁻¹ — the GB300 branch of ``MatrixElements2Band.calc_eps``.

``chi0_eps`` runs pygw.py:3061-3271 on the GPU: the k loop of weighted
Hermitian rank-P updates (pygw.py:3083-3200), then symmetrise, +1, invert,
q→0 head/wings, −1 (pygw.py:3229-3271).  Matrix elements are streamed from
the host (or taken from the device) one k-chunk at a time, as the reference
builds ``minm`` one k at a time.

``MatrixElements2Band.calc_eps`` keeps the reference's signature
(pygw.py:3039); its matrix elements come from ``self.calc_minm`` exactly as in
the reference, so a caller that provides ``calc_minm`` (the LAPW code, or the
synthetic generator here) gets the same data flow.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import free_device_bytes, ptr, require_cuda, stream_handle, to_device, workspace

PRECISION = "fp64"      # 'fp64' (plain comparator) or 'mixed' (split-precision tensor-core χ0)
FSPIN = 2.0


class EpsResult:
    def __init__(self, eps, epsw1, epsw2, head, npb, nom):
        self.eps = eps          # torch [nom][N][N] complex128 (ε⁻¹ − 1), Fortran (I,J,ω) storage
        self.epsw1 = epsw1      # torch [nom][N] or None
        self.epsw2 = epsw2
        self.head = head        # torch [nom] or None
        self.npb, self.nom = npb, nom

    def numpy(self):
        """(eps, epsw1, epsw2, head) in the reference's layouts."""
        eps = self.eps.cpu().numpy().transpose(2, 1, 0)          # (N, N, nom), Fortran order
        if self.epsw1 is None:
            return eps, None, None, None
        return (eps, self.epsw1.cpu().numpy().T.copy(), self.epsw2.cpu().numpy().T.copy(),
                self.head.cpu().numpy().copy())


_COPY_STREAMS: dict[int, "torch.cuda.Stream"] = {}


def _copy_stream():
    """One host→device copy stream per device for the life of the process:
    the caching allocator keeps blocks per stream, so a fresh stream per call
    would allocate (and eventually release, synchronising) the staged matrix
    elements anew every call."""
    dev = torch.cuda.current_device()
    st = _COPY_STREAMS.get(dev)
    if st is None:
        st = _COPY_STREAMS[dev] = torch.cuda.Stream(device=dev)
    return st


def _kcw_device(kcw):
    """kcw as a CUDA float64 tensor whose storage is the Fortran order of (nb1, nb2, nkp, nom)."""
    if isinstance(kcw, torch.Tensor):
        return kcw
    if hasattr(kcw, "kcw"):          # WeightsResult
        return kcw.kcw
    a = np.asarray(kcw, dtype=np.float64)
    return to_device(a.transpose(3, 2, 1, 0), torch.float64)


def _launch_chi0(lib, mk, kc, k0, kcw_d, nb1, nb2, nkp, nom, npb, eps, pmd, epsw1, stream, timers, precision,
                 mctx=None):
    sh = stream_handle(stream)
    ev = None
    if timers is not None:
        s = torch.cuda.current_stream() if stream is None else stream
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ev[0].record(s)
    if precision == "fp64":
        rc = lib.pg_chi0_accumulate_f64(ptr(mk), kc, k0, ptr(kcw_d), nb1, nb2, nkp, nom, npb, -FSPIN, ptr(eps),
                                        ptr(pmd), ptr(epsw1) if pmd is not None else None, sh)
        _lib.check(rc, "pg_chi0_accumulate_f64")
    elif precision == "mixed":
        # split-precision χ0 of this k-chunk added to eps; q = 0 wings in FP64
        rc = lib.pg_chi0_mixed_accumulate(ptr(mk), kc, k0, None, None, 0, ptr(kcw_d), nb1, nb2, nkp, nom, npb,
                                          -FSPIN, ptr(eps), 1 if mctx["started"] else 0, ptr(mctx["work"]),
                                          mctx["work"].numel(), int(mctx["wb"]), 0, ptr(mctx["status"]), sh, None)
        _lib.check(rc, "pg_chi0_mixed_accumulate")
        mctx["started"] = True
        if pmd is not None:
            rc = lib.pg_wings_f64(ptr(mk), kc, k0, ptr(kcw_d), nb1, nb2, nkp, nom, npb, -FSPIN, ptr(pmd), ptr(epsw1),
                                  sh)
            _lib.check(rc, "pg_wings_f64")
    else:
        raise ValueError(f"unknown precision {precision!r}")
    if ev is not None:
        ev[1].record(torch.cuda.current_stream() if stream is None else stream)
        timers.append(ev)


def chi0_accumulate(kcw_d, minm, nkp, npb, nb1, nb2, nom, pm_k=None, k_chunk=None, stream=None, eps=None,
                    epsw1=None, precision=None, timers=None, status=None):
    """Σ_k of the weighted rank-P updates into ``eps`` (and ``epsw1`` for q = 0).

    ``minm`` is either a callable ``minm(ik) -> minm[nb1, nb2, npb]`` (numpy or
    tensor, the reference's per-k ``calc_minm``), or a complex128 tensor
    ``[nkp, P, npb]`` — on the device (used in place) or in pinned host memory
    (streamed in k-chunks on a side stream, double-buffered against the
    contraction).  ``pm_k(ik)`` returns the q→0 vector ``pm[P]``.
    ``precision='mixed'`` runs the split-precision tensor-core contraction per
    k-chunk (``status``, a device int32 tensor, receives its PG_ERR_* bits).
    ``timers`` (a list) receives a CUDA event pair around each χ0 launch.
    """
    precision = precision or PRECISION
    lib = _lib.load()
    P = nb1 * nb2
    cur = torch.cuda.current_stream() if stream is None else stream
    if eps is None:
        eps = torch.zeros((nom, npb, npb), dtype=torch.complex128, device="cuda")
    if pm_k is not None and epsw1 is None:
        epsw1 = torch.zeros((nom, npb), dtype=torch.complex128, device="cuda")
    on_device = isinstance(minm, torch.Tensor) and minm.is_cuda
    # Pinned host matrix elements for the split-precision contraction are
    # staged whole when they fit: one copy, started while the weights kernel
    # may still be running, then one pass over all k (per-chunk passes repeat
    # the digit preparation and run shorter GEMM launches).
    staged = False
    if not on_device and k_chunk is None and precision == "mixed" and isinstance(minm, torch.Tensor):
        free = free_device_bytes()
        wb_all = mixed_omega_batch(nb1, nb2, nkp, npb, nom)
        need = nkp * P * npb * 16 + lib.pg_chi0_mixed_workspace(nb1, nb2, nkp, npb, wb_all, 0)
        staged = need <= 0.8 * free
    if on_device or staged:
        k_chunk = nkp                    # resident: one pass over all k
    elif k_chunk is None:
        # the tensor-core contraction wants long K per launch: bigger chunks
        budget = (4 << 30) if precision == "mixed" else (256 << 20)
        k_chunk = max(1, min(nkp, budget // max(1, P * npb * 16)))
    mctx = None
    if precision == "mixed":
        kc_max = min(k_chunk, nkp)
        wb = mixed_omega_batch(nb1, nb2, kc_max, npb, nom)
        mctx = {"wb": wb, "started": False,
                "work": workspace(lib.pg_chi0_mixed_workspace(nb1, nb2, kc_max, npb, wb, 0)),
                "status": status if status is not None else torch.zeros(1, dtype=torch.int32, device="cuda")}

    def pm_chunk(k0, kc):
        if pm_k is None:
            return None
        return to_device(np.stack([np.asarray(pm_k(ik), dtype=np.complex128) for ik in range(k0, k0 + kc)]),
                         torch.complex128)

    if on_device:
        m = minm.reshape(nkp, P, npb)
        _launch_chi0(lib, m, nkp, 0, kcw_d, nb1, nb2, nkp, nom, npb, eps, pm_chunk(0, nkp), epsw1, stream, timers,
                     precision, mctx)
        return eps, epsw1

    if staged:
        copy_stream = _copy_stream()
        # allocated on the copy stream: its memory is none that kernels still
        # queued on the compute stream use, so the copy need not wait for them
        with torch.cuda.stream(copy_stream):
            dev = torch.empty((nkp, P, npb), dtype=torch.complex128, device="cuda")
            dev.copy_(minm.reshape(nkp, P, npb), non_blocking=True)
            done = torch.cuda.Event()
            done.record(copy_stream)
        dev.record_stream(cur)
        cur.wait_event(done)
        _launch_chi0(lib, dev, nkp, 0, kcw_d, nb1, nb2, nkp, nom, npb, eps, pm_chunk(0, nkp), epsw1, stream, timers,
                     precision, mctx)
        return eps, epsw1

    if isinstance(minm, torch.Tensor):
        # pinned host tensor: double-buffered H2D on a copy stream
        m = minm.reshape(nkp, P, npb)
        bufs = [torch.empty((k_chunk, P, npb), dtype=torch.complex128, device="cuda") for _ in range(2)]
        copy_stream = _copy_stream()
        # The buffers come from the caching allocator of the compute stream and
        # may reuse memory that kernels still queued there (e.g. the weight
        # kernel's workspace) are using: the copy stream starts after them, and
        # the allocator is told the buffers are also used on the copy stream.
        copy_stream.wait_stream(cur)
        for b in bufs:
            b.record_stream(copy_stream)
        copied = [torch.cuda.Event() for _ in range(2)]
        used = [None, None]
        for i, k0 in enumerate(range(0, nkp, k_chunk)):
            kc = min(k_chunk, nkp - k0)
            b = i % 2
            with torch.cuda.stream(copy_stream):
                if used[b] is not None:
                    copy_stream.wait_event(used[b])
                bufs[b][:kc].copy_(m[k0:k0 + kc], non_blocking=True)
                copied[b].record(copy_stream)
            cur.wait_event(copied[b])
            _launch_chi0(lib, bufs[b], kc, k0, kcw_d, nb1, nb2, nkp, nom, npb, eps, pm_chunk(k0, kc), epsw1, stream,
                         timers, precision, mctx)
            used[b] = torch.cuda.Event()
            used[b].record(cur)
        return eps, epsw1

    for k0 in range(0, nkp, k_chunk):
        kc = min(k_chunk, nkp - k0)
        blocks = []
        for ik in range(k0, k0 + kc):
            mm = minm(ik)
            if isinstance(mm, torch.Tensor):
                blocks.append(mm.reshape(P, npb).to(torch.complex128))
            else:
                blocks.append(torch.from_numpy(np.ascontiguousarray(mm, dtype=np.complex128).reshape(P, npb)))
        mk = torch.stack(blocks)
        mk = mk if mk.is_cuda else mk.cuda()
        _launch_chi0(lib, mk, kc, k0, kcw_d, nb1, nb2, nkp, nom, npb, eps, pm_chunk(k0, kc), epsw1, stream, timers,
                     precision, mctx)
    return eps, epsw1


def _all_k_device(minm, nkp, P, npb):
    """Matrix elements of every k as one CUDA tensor [nkp, P, npb] (complex128)."""
    if isinstance(minm, torch.Tensor):
        m = minm.reshape(nkp, P, npb)
        return m if m.is_cuda else m.cuda(non_blocking=True)
    out = torch.empty((nkp, P, npb), dtype=torch.complex128, device="cuda")
    for ik in range(nkp):
        mm = minm(ik)
        t = mm if isinstance(mm, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(mm, dtype=np.complex128))
        out[ik].copy_(t.reshape(P, npb))
    return out


def mixed_omega_batch(nb1, nb2, nkp, npb, nom, budget_bytes=None, sm_count=None):
    """Frequencies per launch of the split-precision χ0: the fewest that give
    the digit GEMM two waves of 2-CTA clusters, within a memory budget
    (default: 40 % of the free device memory).  Fewer frequencies per launch
    leave more of L2 to the digit planes they share: at N_PB 1200 and 6³ k one
    frequency per launch reads 427 GB from DRAM per frequency, two 525 GB, four
    567 GB, and runs 7 % faster than two.  ``sm_count`` defaults to the
    current device's."""
    lib = _lib.load()
    if budget_bytes is None:
        free = free_device_bytes()
        budget_bytes = int(0.4 * free)
    if sm_count is None:
        sm_count = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    clusters = max(1, sm_count // 2)
    offs = (ctypes.c_size_t * 9)()
    dims = (ctypes.c_longlong * 9)()
    wb = 1
    while wb < nom and lib.pg_chi0_mixed_workspace(nb1, nb2, nkp, npb, 2 * wb, 0) <= budget_bytes:
        _lib.check(lib.pg_chi0_mixed_layout(nb1, nb2, nkp, npb, wb, 0, offs, dims), "pg_chi0_mixed_layout")
        nc = dims[3] // 256
        if nc * (nc + 1) // 2 * wb * dims[7] >= 2 * clusters:
            break
        wb *= 2
    return min(wb, nom)


def chi0_mixed(kcw_d, minm, nkp, npb, nb1, nb2, nom, omega_batch=None, kb_split=0, stream=None, work=None,
               timers=None, gemm_timers=None):
    """Split-precision χ0 (tensor cores) for all frequencies: returns
    ``(eps, status, work)`` with the full Hermitian χ0 in ``eps`` [nom][N][N].
    ``timers`` receives one (start, end) event pair around the whole call,
    ``gemm_timers`` one pair per frequency batch around the digit-GEMM kernel."""
    lib = _lib.load()
    P = nb1 * nb2
    m = _all_k_device(minm, nkp, P, npb)
    wb = omega_batch or mixed_omega_batch(nb1, nb2, nkp, npb, nom)
    wbytes = lib.pg_chi0_mixed_workspace(nb1, nb2, nkp, npb, wb, int(kb_split))
    if work is None or work.numel() < wbytes:
        work = workspace(wbytes)
    eps = torch.empty((nom, npb, npb), dtype=torch.complex128, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream() if stream is None else stream
    ev = None
    if timers is not None:
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ev[0].record(s)
    gev = None
    if gemm_timers is not None:
        nbatch = -(-nom // min(wb, nom))
        gev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * nbatch)]
        for e in gev:
            e.record(s)                          # creates the CUDA event behind each object
        handles = (ctypes.c_void_p * len(gev))(*[e.cuda_event for e in gev])
    rc = lib.pg_chi0_mixed(ptr(m), nkp, ptr(kcw_d), nb1, nb2, nom, npb, -FSPIN, ptr(eps), ptr(work), work.numel(),
                           int(wb), int(kb_split), ptr(status), stream_handle(stream),
                           handles if gev is not None else None)
    _lib.check(rc, "pg_chi0_mixed")
    if ev is not None:
        ev[1].record(s)
        timers.append(ev)
    if gev is not None:
        gemm_timers.extend((gev[2 * b], gev[2 * b + 1]) for b in range(len(gev) // 2))
    return eps, status, work


def wings_f64(kcw_d, minm, nkp, npb, nb1, nb2, nom, pm_k, stream=None):
    """q→0 wings ``epsw1[ω][I]`` in FP64 (pygw.py:3192-3195)."""
    lib = _lib.load()
    P = nb1 * nb2
    m = _all_k_device(minm, nkp, P, npb)
    pmd = to_device(np.stack([np.asarray(pm_k(ik), dtype=np.complex128) for ik in range(nkp)]), torch.complex128)
    epsw1 = torch.zeros((nom, npb), dtype=torch.complex128, device="cuda")
    rc = lib.pg_wings_f64(ptr(m), nkp, 0, ptr(kcw_d), nb1, nb2, nkp, nom, npb, -FSPIN, ptr(pmd), ptr(epsw1),
                          stream_handle(stream))
    _lib.check(rc, "pg_wings_f64")
    return epsw1


def chi0_finalize(eps, npb, nom, stream=None, precision=None):
    lib = _lib.load()
    rc = lib.pg_chi0_mirror_f64(ptr(eps), npb, nom, stream_handle(stream))
    _lib.check(rc, "pg_chi0_mirror_f64")
    return eps


REFINE_ITERS = 2       # refinement steps of the mixed-precision inverse (0 = FP32 inverse alone)


def eps_inverse_batch(npb, nom, budget_bytes=None):
    """Frequencies per batch of the mixed-precision inverse, sized to a memory
    budget (default: 30 % of the free device memory)."""
    lib = _lib.load()
    if budget_bytes is None:
        free = free_device_bytes()
        budget_bytes = int(0.3 * free)
    nb = nom
    while nb > 1 and lib.pg_eps_inverse_mixed_workspace(npb, nom, nb) > budget_bytes:
        nb = (nb + 1) // 2
    return nb


def eps_inverse(eps, npb, nom, epsw1=None, head=None, stream=None, precision=None, work=None, iters=None,
                omega_batch=None):
    """ε⁻¹ − 1 in place; for q = 0 also the updated wings and head.

    ``precision='mixed'``: FP32 inverse refined ``iters`` times in FP64 with the
    residual on the tensor cores (``pg_eps_inverse_mixed``); otherwise the FP64
    Gauss–Jordan inverse (``pg_eps_inverse_f64``)."""
    lib = _lib.load()
    precision = precision or PRECISION
    epsw2 = None
    head_d = None
    if epsw1 is not None:
        epsw2 = torch.conj(epsw1).resolve_conj().contiguous()
        head_d = to_device(np.asarray(head, dtype=np.complex128), torch.complex128).clone()
    status = None
    if precision == "mixed":
        nb = omega_batch or eps_inverse_batch(npb, nom)
        wb = lib.pg_eps_inverse_mixed_workspace(npb, nom, nb)
        if work is None or work.numel() < wb:
            work = workspace(wb)
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        rc = lib.pg_eps_inverse_mixed(ptr(eps), npb, nom, ptr(epsw1), ptr(epsw2), ptr(head_d), ptr(work),
                                      work.numel(), int(nb), int(REFINE_ITERS if iters is None else iters),
                                      ptr(status), stream_handle(stream))
        _lib.check(rc, "pg_eps_inverse_mixed")
    else:
        wb = lib.pg_eps_inverse_f64_workspace(npb, nom)
        if work is None or work.numel() < wb:
            work = workspace(wb)
        rc = lib.pg_eps_inverse_f64(ptr(eps), npb, nom, ptr(epsw1), ptr(epsw2), ptr(head_d), ptr(work),
                                    work.numel(), stream_handle(stream))
        _lib.check(rc, "pg_eps_inverse_f64")
    r = EpsResult(eps, epsw1, epsw2, head_d, npb, nom)
    r.status = status
    return r


def chi0_eps(kcw, minm, nkp, npb, nb1, nb2, nom, pm_k=None, head=None, k_chunk=None, stream=None, precision=None,
             timers=None, Ul=None, dUl=None):
    """The whole ε path for one q on the GPU: returns an ``EpsResult``.

    ``minm``: per-k callable or ``[nkp, P, npb]`` tensor (see chi0_accumulate).
    With the SVD frequency basis (``Ul`` (nl, nω), ``dUl`` (nω, nl)), ``kcw``
    holds par3 weights, ``nom`` is nl and ``head`` is given in the basis; χ0 is
    accumulated on the nl basis functions, ε, its wings and head go to
    frequencies with Ul for the inverse and back with dUl (pygw.py:3043-3045,
    3204-3226, 3274-3280)."""
    require_cuda()
    kcw_d = _kcw_device(kcw)
    precision = precision or PRECISION
    status = None
    if precision == "mixed":
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        eps, epsw1 = chi0_accumulate(kcw_d, minm, nkp, npb, nb1, nb2, nom, pm_k=pm_k, k_chunk=k_chunk, stream=stream,
                                     precision="mixed", timers=timers, status=status)
    else:
        eps, epsw1 = chi0_accumulate(kcw_d, minm, nkp, npb, nb1, nb2, nom, pm_k=pm_k, k_chunk=k_chunk, stream=stream,
                                     precision=precision, timers=timers)
        chi0_finalize(eps, npb, nom, stream=stream, precision=precision)
    if Ul is None:
        r = eps_inverse(eps, npb, nom, epsw1=epsw1, head=head, stream=stream, precision=precision)
        r.chi0_status = status
        return r
    from .svd import to_basis
    Ul = np.asarray(Ul, dtype=np.float64)
    dUl = np.asarray(dUl, dtype=np.float64)
    eps_w = to_basis(eps, Ul, stream=stream)
    epsw1_w = to_basis(epsw1, Ul, stream=stream) if epsw1 is not None else None
    head_w = None if head is None else np.dot(np.asarray(head, dtype=complex), Ul)
    nw = Ul.shape[1]
    r = eps_inverse(eps_w, npb, nw, epsw1=epsw1_w, head=head_w, stream=stream, precision=precision)
    out = EpsResult(to_basis(r.eps, dUl, stream=stream),
                    to_basis(r.epsw1, dUl, stream=stream) if r.epsw1 is not None else None,
                    to_basis(r.epsw2, dUl, stream=stream) if r.epsw2 is not None else None,
                    to_basis(r.head.reshape(nw, 1), dUl, stream=stream).reshape(-1) if r.head is not None else None,
                    npb, Ul.shape[0])
    out.status = r.status
    out.chi0_status = status
    return out


def momentum_vectors(head_quantities, ks, core, kqm, vol, isp=0):
    """The q→0 vectors ``pm[ik, (ncg_p + nvbm)·nb2]`` that calc_eps forms from
    the momentum matrix elements in ``head_quantities = (head, mmatcv,
    mmatvv, mst)`` (pygw.py:3120-3141), core states first: for each
    (occupied or core, empty) pair the x + y + z sum of ⟨p⟩ (stored from band
    ``mst`` on) times 2√(π/Vol)/√3, divided by the energy difference, or 0
    where the two energies are within 1e-10.  The energies are the core
    levels ``core.eig_core[isp][iat][ic]`` of ``core.corind`` and the bands
    of the irreducible k point (pygw.py:3089-3093).  Host-side argument
    assembly: a few thousand entries per k point."""
    _, mmatcv, mmatvv, mst = head_quantities
    nvbm, ncbm = ks.nomax_numin[0] + 1, ks.nomax_numin[1]
    nbmax, ncg = ks.nbmaxpol, ks.ncg_p
    coefw = 2.0 * np.sqrt(np.pi / vol)
    scale = coefw / np.sqrt(3.0)
    corind = np.asarray(core.corind)
    ecore = np.array([core.eig_core[isp][int(iat)][int(ic)] for iat, _, ic in corind[:ncg, :3]], dtype=np.float64)
    pm = np.zeros((len(kqm.kii_ind), (ncg + nvbm) * (nbmax - ncbm)), dtype=np.complex128)
    for ik, irk in enumerate(kqm.kii_ind):
        eb = np.asarray(ks.Ebnd[isp, irk, :nbmax], dtype=np.float64)
        mmc = np.sum(mmatcv[irk, ncbm - mst:nbmax - mst, :, :], axis=2) * scale    # [nb2, ncg]
        mmv = np.sum(mmatvv[irk, ncbm - mst:nbmax - mst, :, :], axis=2) * scale    # [nb2, nvbm]
        rows = []
        for e1, m in ((ecore, mmc[:, :ncg]), (eb[:nvbm], mmv[:, :nvbm])):
            edif = e1[:, None] - eb[None, ncbm:nbmax]
            big = np.abs(edif) > 1e-10
            r = np.zeros(edif.shape, dtype=np.complex128)
            r[big] = m.T[big] / edif[big]
            rows.append(r)
        pm[ik] = np.concatenate(rows, axis=0).ravel()
    return pm


class MatrixElements2Band:
    """Stand-in for the reference class with the GB300 ``calc_eps`` and ``calc_selfc``.

    ``calc_minm(ik, iq, band_limits, mode, ...)`` must return
    ``(minm0, minc0)`` as in the reference (pygw.py:3096-3098 for
    'polarization', 3342-3349 for 'selfe'); the synthetic generator provides
    one (``synthetic_matrix_elements``).  singc1/singc2 are the q→0
    singularity coefficients calc_selfc uses at q = 0 (pygw.py:3310-3311).
    At q = 0 calc_eps forms the wings' vectors from ``head_quantities`` as
    the reference does (``momentum_vectors``) unless ``pm_k(ik)`` is given
    here, which then supplies them directly (the synthetic workloads draw
    them per k point).
    """

    def __init__(self, calc_minm, matsize, pm_k=None, singc1=0.0, singc2=0.0):
        self.calc_minm = calc_minm
        self.matsize = matsize
        self.pm_k = pm_k
        self.singc1, self.singc2 = singc1, singc2

    def calc_eps(self, iq, head_quantities, strc, in1, latgen, kqm, ks, radf, pw, pb, core, kw, fr, kcw, ddir, dUl,
                 Ul, fout):
        nvbm, ncbm = ks.nomax_numin[0] + 1, ks.nomax_numin[1]
        nb1, nb2 = ks.ncg_p + nvbm, ks.nbmaxpol - ncbm
        nkp = len(kqm.kii_ind)
        # with the SVD basis kcw (par3) and the outputs carry nl basis functions
        nom = len(fr.omega) if Ul is None else np.asarray(Ul).shape[0]
        band_limits = (0, nvbm, ncbm, ks.nbmaxpol, 0, ks.ncg_p)

        def minm_k(ik):
            minm0, minc0 = self.calc_minm(ik, iq, band_limits, "polarization")
            return minm0 if minc0 is None else np.concatenate((minc0, minm0), axis=0)

        head = pm_k = None
        if iq == 0:
            head = head_quantities[0]
            pm_k = self.pm_k
            if pm_k is None:
                pm = momentum_vectors(head_quantities, ks, core, kqm, latgen.Vol)
                pm_k = pm.__getitem__
        r = chi0_eps(kcw, minm_k, nkp, self.matsize, nb1, nb2, nom, pm_k=pm_k, head=head, Ul=Ul, dUl=dUl)
        eps, epsw1, epsw2, head_out = r.numpy()
        if fout is not None:
            for iom in range(eps.shape[2]):
                print("Tr(1/eps[%3d]-1) = %18.14f" % (iom + 1, np.trace(eps[:, :, iom]).real), file=fout)
        return eps, epsw1, epsw2, head_out

    def calc_selfc(self, iq, eps, epsw1, epsw2, head, strc, in1, latgen, kqm, ks, radf, pw, pb, core, kw, fr, ddir,
                   dUl, Ul, fout, PRINT=True):
        """pygw.py:3299 — Σc contributions sc_p[nirkp, nbgw − ibgw, nom] of this q (see selfc.calc_selfc)."""
        from .selfc import calc_selfc
        return calc_selfc(self, iq, eps, epsw1, epsw2, head, strc, in1, latgen, kqm, ks, radf, pw, pb, core, kw, fr,
                          ddir, dUl, Ul, fout, PRINT=PRINT)
