#!/usr/bin/env python
"""Seconds per q-point of PyGW's polarization path — weights → χ0 → ε⁻¹ — on GB300.

One step = one q-point of the workload: tetrahedron weights w_nm(k,q,iω), the
χ0 contraction over all k, the symmetrised dielectric matrix and its inverse
per frequency.  ``value`` is measured with every input already resident in
HBM; ``e2e`` runs the same step through the package's public Python API from
pinned host buffers (matrix elements streamed host→device per k-chunk) and
reads ε⁻¹−1 back to the host.  Inputs are seeded synthetic data with the
workload's shapes (no public dataset is involved).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload C2] [--impl gb300|reference]

With N > 1 (torchrun) every rank is an independent replica over its own q
points (the reference splits q over MPI ranks with no collective on this path);
the timed region is bracketed by barriers and the maximum over ranks is kept.
``--impl reference`` times the reference's CPU implementation of the path
(the oracle's restatement: C++/OpenMP weights + numpy contraction and
inverse) on the host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="C3")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--prep-batch", type=int, default=0,
                    help="split-precision chi0: frequencies per B-digit preparation pass (0: the library default)")
    ap.add_argument("--fp64-k-sample", type=int, default=4,
                    help="k-points on which the plain FP64 GPU contraction is timed for the comparison line")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="mixed: skip the FP64-vs-mixed eps^-1 comparison on three frequencies (outside the timed "
                         "region)")
    ap.add_argument("--div", type=int, default=0, help="override the k-mesh divisions (smaller profiling case)")
    ap.add_argument("--npb", type=int, default=0, help="override the product-basis size (smaller profiling case)")
    ap.add_argument("--nom", type=int, default=0, help="override the number of frequencies (smaller profiling case)")
    ap.add_argument("--q-limit", type=int, default=0, help="batched workloads: only the first n q points")
    ap.add_argument("--no-tune", action="store_true", help="batched workloads: default work split, no autotuning")
    ap.add_argument("--no-graph", action="store_true", help="batched workloads: enqueue eagerly, no CUDA graph")
    ap.add_argument("--tune-file", default=None, help="batched workloads: JSON file the autotuner reads and extends")
    ap.add_argument("--path", default="polarization", choices=["polarization", "selfc"],
                    help="selfc: the correlation self-energy step (mwm contraction + Matsubara convolution) "
                         "on the workload's k mesh, N_PB and frequencies")
    ap.add_argument("--selfc-nb1", type=int, default=16, help="selfc: GW bands (nbgw - ibgw)")
    ap.add_argument("--omega-batch", type=int, default=0,
                    help="mixed chi0: frequencies per digit-GEMM launch (0: the library's rule)")
    ap.add_argument("--kb-split", type=int, default=0,
                    help="mixed chi0: K-blocks per K split of the digit GEMM (0: automatic)")
    return ap.parse_args()


def workload_desc(w):
    return (f"{w.name}: {w.div}^3 k-mesh ({6 * w.div ** 3} tetrahedra), {w.nbands} bands ({w.nocc} occ), "
            f"N_PB={w.npb}, {w.nom} log-spaced iw in {w.om_lo}-{w.om_hi} eV, {w.nq} q")


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons.

    The sampler process is started before this process initialises CUDA (no
    fork of a process that holds a CUDA context) and runs for the whole
    bench; ``window(t0, t1)`` summarises the samples taken inside a timed
    region (host wall-clock times)."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def window(self, t0, t1):
        if self.path is None or not os.path.exists(self.path):
            return None
        import datetime
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                clk, mx = float(parts[2]), float(parts[3])
            except ValueError:
                continue
            if not (t0 - 0.25 <= ts <= t1 + 0.25):
                continue
            sm.append(clk)
            smax.append(mx)
            for n, v in zip(names, parts[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}

    def cleanup(self):
        if self.path and os.path.exists(self.path):
            os.unlink(self.path)


# --------------------------------------------------------------- problem
class Inputs:
    """Host and device inputs of one workload (matrix elements of one q reused).

    Every host buffer the e2e path copies from, and the buffer it reads the
    result into, is pinned here once, before any GPU work; the timed loops
    issue no pageable copies."""

    def __init__(self, w, rank, device_resident=True):
        import torch

        from pygw_gb300 import synthetic as syn
        self.w = w
        self.p = syn.Problem(w)
        b = self.p.bands
        self.nomx, self.numin = b.nomax_numin
        self.nb1, self.nb2 = b.nb1, b.nb2
        self.P = self.nb1 * self.nb2
        self.nkp = self.p.kqm.nkp
        self.enk = b.enk()
        self.ef = b.EF
        self.omega = self.p.fr.omega
        self.tetc = self.p.kqm.tetc
        self.kqid = self.p.kqm.kqid
        self.qs = self.p.qs
        iq0 = self.qs[0]
        sqv = syn.coulomb_sqrt(w, iq0, w.npb)
        self.minm_host = torch.empty((self.nkp, self.P, w.npb), dtype=torch.complex128).pin_memory()
        for ik in range(self.nkp):
            m = syn.minm_k(w, b, self.p.kqm, iq0, ik, sqv).reshape(self.P, w.npb)
            self.minm_host[ik].copy_(torch.from_numpy(m))
        # pinned host copies in the C-ABI layouts
        self.enk_h = torch.from_numpy(np.ascontiguousarray(self.enk.T)).pin_memory()                # [nkp][nbnd]
        self.tetc_h = torch.from_numpy(np.ascontiguousarray(self.tetc.T.astype(np.int32))).pin_memory()
        self.kqid_h = torch.from_numpy(np.ascontiguousarray(self.kqid.T.astype(np.int32))).pin_memory()  # [iq][ik]
        self.om_h = torch.from_numpy(self.omega.copy()).pin_memory()
        self.out_h = torch.empty((w.nom, w.npb, w.npb), dtype=torch.complex128).pin_memory()
        torch.cuda.synchronize()
        self.minm_dev = self.minm_host.cuda() if device_resident else None
        self.enk_d = self.enk_h.cuda()
        self.tetc_d = self.tetc_h.cuda()
        self.kqid_d = self.kqid_h.cuda()
        self.om_d = self.om_h.cuda()
        torch.cuda.synchronize()


def gpu_step(inp, step, timers=None, stream=None, precision="fp64", phases=None):
    """One q-point with device-resident inputs; ``phases`` (a list) receives
    CUDA events bracketing weights / χ0 / ε⁻¹."""
    import torch
    from pygw_gb300 import eps as peps
    from pygw_gb300 import polarization as pol
    iq = inp.qs[step % len(inp.qs)]
    cs = torch.cuda.current_stream() if stream is None else stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if phases is not None else None
    if ev:
        ev[0].record(cs)
    r = pol.weights_device(inp.enk_d, inp.ef, inp.kqid_d[iq], 0, inp.nomx, inp.numin, inp.om_d, inp.tetc_d,
                           stream=stream)
    if ev:
        ev[1].record(cs)
    if precision == "mixed":
        eps, status, inp.mwork = peps.chi0_mixed(r.kcw, inp.minm_dev, inp.nkp, inp.w.npb, inp.nb1, inp.nb2,
                                                 inp.w.nom, omega_batch=inp.wb, kb_split=inp.kb_split, stream=stream,
                                                 work=getattr(inp, "mwork", None), timers=timers,
                                                 gemm_timers=inp.gemm_timers if timers is not None else None)
        inp.statuses.append(status)
    else:
        eps, _ = peps.chi0_accumulate(r.kcw, inp.minm_dev, inp.nkp, inp.w.npb, inp.nb1, inp.nb2, inp.w.nom,
                                      stream=stream, timers=timers)
        peps.chi0_finalize(eps, inp.w.npb, inp.w.nom, stream=stream)
    if ev:
        ev[2].record(cs)
    res = peps.eps_inverse(eps, inp.w.npb, inp.w.nom, stream=stream, precision=precision)
    if precision == "mixed":
        inp.statuses.append(res.status)
    if ev:
        ev[3].record(cs)
        phases.append(ev)
    return res


def fp64_gpu_estimate(inp, nk):
    """Seconds per q-point of the plain FP64 GPU path: weights and ε⁻¹ timed in
    full, the FP64 contraction timed on ``nk`` k-points and scaled to all k."""
    import torch
    from pygw_gb300 import _lib
    from pygw_gb300 import eps as peps
    from pygw_gb300 import polarization as pol
    from pygw_gb300.device import ptr, stream_handle
    lib = _lib.load()
    nk = max(1, min(nk, inp.nkp))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    cs = torch.cuda.current_stream()
    iq = inp.qs[0]
    ev[0].record(cs)
    r = pol.weights_device(inp.enk_d, inp.ef, inp.kqid_d[iq], 0, inp.nomx, inp.numin, inp.om_d, inp.tetc_d)
    ev[1].record(cs)
    eps = torch.zeros((inp.w.nom, inp.w.npb, inp.w.npb), dtype=torch.complex128, device="cuda")
    rc = lib.pg_chi0_accumulate_f64(ptr(inp.minm_dev), nk, 0, ptr(r.kcw), inp.nb1, inp.nb2, inp.nkp, inp.w.nom,
                                    inp.w.npb, -2.0, ptr(eps), None, None, stream_handle(None))
    _lib.check(rc, "pg_chi0_accumulate_f64")
    peps.chi0_finalize(eps, inp.w.npb, inp.w.nom)
    ev[2].record(cs)
    peps.eps_inverse(eps, inp.w.npb, inp.w.nom, precision="fp64")
    ev[3].record(cs)
    torch.cuda.synchronize()
    t_w = ev[0].elapsed_time(ev[1]) * 1e-3
    t_c = ev[1].elapsed_time(ev[2]) * 1e-3 * inp.nkp / nk
    t_i = ev[2].elapsed_time(ev[3]) * 1e-3
    return t_w + t_c + t_i, {"weights_s": t_w, "chi0_s": t_c, "eps_inverse_s": t_i,
                             "sample": f"FP64 contraction timed on {nk}/{inp.nkp} k-points and scaled"}


def e2e_step(inp, step, out_host, precision="fp64"):
    """One q-point through the public API from pinned host buffers; result read back."""
    from pygw_gb300 import eps as peps
    from pygw_gb300 import polarization as pol
    iq = inp.qs[step % len(inp.qs)]
    r = pol.weights_device(inp.enk_h, inp.ef, inp.kqid_h[iq], 0, inp.nomx, inp.numin, inp.om_h, inp.tetc_h)
    res = peps.chi0_eps(r, inp.minm_host, inp.nkp, inp.w.npb, inp.nb1, inp.nb2, inp.w.nom, precision=precision)
    out_host.copy_(res.eps, non_blocking=True)
    return res


def mixed_tile_area(npb):
    """Output elements the digit GEMM computes per frequency and K: 256x256
    blocks of the upper block triangle of the 2N x 2N product (k_ozaki_gemm,
    one 2-SM MMA per block and 16 K)."""
    nc = -(-2 * npb // 256)
    return nc * (nc + 1) // 2 * 256 * 256


def bf16_peak():
    """The bf16 denominator for a kernel timed inside a multi-second step: the
    measured sustained figure (the burst one is for a kernel timed alone)."""
    peaks = json.load(open(PEAKS_FILE)) if os.path.exists(PEAKS_FILE) else {}
    if "bf16_tflops_sustained" in peaks:
        return peaks["bf16_tflops_sustained"], "of measured (sustained)"
    if "bf16_tflops" in peaks:
        return peaks["bf16_tflops"], "of measured (burst)"
    return 1700.0, "of fallback (sustained)"


# DRAM bytes (read + written) of one launch of the χ0 digit GEMM, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) per kernel build and
# launch shape: (kernel, workload, N_PB, k-points, frequencies per launch) ->
# (bytes, where the capture is summarised).  A launch whose kernel or shape has
# no entry reports traffic null and says so.
GEMM_BUILD = "k_ozaki_gemm 2-SM M256 N256, 6 stages"
MEASURED_GEMM_TRAFFIC = {
    (GEMM_BUILD, "C3", 1200, 216, 1): (287.65e9 + 0.59e9, "profiles/k_ozaki_gemm_2sm_c3_dram_traffic.md"),
}


# FP64 work of the weight kernels and the FP64 ceiling it is held to, from one
# ncu capture of k_tet_geometry, k_tet_eval and k_chi0_f64 (thread-level dadd,
# dmul, dfma instruction counts, FP64-pipe instructions, gpu__time_duration):
# (FP64 flops (dadd + dmul + 2·dfma) per (sub-tetrahedron, ω) evaluation,
# geometry included, counted by the kernels' exact + Taylor counters;
# k_chi0_f64's FP64 rate in TFLOP/s with its FP64 pipe 97 % busy; FP64-pipe
# thread instructions per evaluation (flop-type and the rest: comparisons,
# conversions); k_chi0_f64's FP64-pipe thread-instruction rate; where the
# capture is summarised).  The weights mix single-flop adds and multiplies
# and non-flop FP64 instructions into their FMAs, so they keep the FP64 pipe
# busy at a lower flop rate than the FMA-only contraction.
WEIGHTS_FP64 = (308.9, 1.212, 316.0, 0.6112e12, "profiles/fp64_work_k_tet_geometry_eval_k_chi0_f64_c2_div4.md")


def measure_accuracy(inp):
    """Split-precision ε⁻¹ of the benchmarked q against the FP64 GPU path, on
    the lowest, a middle and the highest frequency, with every k-point
    (outside the timed region)."""
    from pygw_gb300 import accuracy
    from pygw_gb300 import polarization as pol
    iq = inp.qs[0]
    r = pol.weights_device(inp.enk_d, inp.ef, inp.kqid_d[iq], 0, inp.nomx, inp.numin, inp.om_d, inp.tetc_d)
    nom = inp.w.nom
    t0 = time.perf_counter()
    acc = accuracy.mixed_vs_fp64(r.kcw, inp.minm_dev, inp.nkp, inp.w.npb, inp.nb1, inp.nb2,
                                 sorted({0, nom // 2, nom - 1}))
    acc["seconds"] = time.perf_counter() - t0
    acc["note"] = ("eps^-1 of the benchmarked q from the split-precision path vs the FP64 GPU path, same weights and "
                   "matrix elements, all k-points; normwise = max|d|/max|ref| (the 1e-9 bar), elementwise = "
                   "max|d_ij|/|ref_ij| over |ref_ij| > elementwise_floor*max|ref|")
    return acc


def weights_roofline(inp):
    """Roofline of the weights phase of one q (the first): the kcw bytes it
    writes against the HBM copy bandwidth, and its FP64 work (from the
    kernel's own evaluation counters) against the FP64 ceiling of the plain
    FP64 contraction.  Timed with CUDA events around the phase (warm)."""
    import torch
    from pygw_gb300 import polarization as pol
    iq = inp.qs[0]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ts = []
    for _ in range(3):
        ev[0].record()
        r = pol.weights_device(inp.enk_d, inp.ef, inp.kqid_d[iq], 0, inp.nomx, inp.numin, inp.om_d, inp.tetc_d)
        ev[1].record()
        torch.cuda.synchronize()
        ts.append(ev[0].elapsed_time(ev[1]))
    t_ms = statistics.median(ts)
    c = r.counters
    nom = inp.w.nom
    kcw_bytes = 8 * inp.nb1 * inp.nb2 * inp.nkp * nom
    hbm = json.load(open(PEAKS_FILE)).get("hbm_gbs") if os.path.exists(PEAKS_FILE) else 6800.0
    gbs = kcw_bytes / (t_ms * 1e-3) / 1e9
    out = {"kernel": "weights phase (k lists, k_tet_geometry, k_class_scatter, k_tet_eval, k_gather)",
           "phase_ms": t_ms, "evaluations": {"exact": c["exact"], "taylor": c["taylor"], "calls": c["calls"]},
           "hbm": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                   "algorithmic_bytes": kcw_bytes, "note": "kcw written (8 B per band pair, k-point, frequency) / "
                                                          "phase time; peak = measured copy bandwidth"},
           "fp64": None}
    if WEIGHTS_FP64 is not None:
        per_eval, ceiling, instr_per_eval, instr_ceiling, src = WEIGHTS_FP64
        nev = c["exact"] + c["taylor"]
        flops = per_eval * nev
        tf = flops / (t_ms * 1e-3) / 1e12
        ips = instr_per_eval * nev / (t_ms * 1e-3)
        out["fp64"] = {"bound": "fp64", "achieved": tf, "peak": ceiling, "unit": "TFLOP/s", "frac": tf / ceiling,
                       "flops": flops, "source": src,
                       "pipe_frac": ips / instr_ceiling,
                       "note": "FP64 flops = per-evaluation count (dadd + dmul + 2 dfma) x (exact + Taylor "
                               "evaluations of this q); peak = FP64 rate of this build's k_chi0_f64 (FP64 pipe "
                               "97 % busy); pipe_frac = FP64-pipe instructions per evaluation x evaluations / "
                               "phase time / k_chi0_f64's FP64-pipe instruction rate"}
    return out


# GB300's FP64 rate (CUDA cores; it has no faster FP64 tensor path).  The
# measured peaks file holds HBM and bf16 figures only, so the FP64 roofline
# of the plain path is quoted against this nominal figure.
FP64_NOMINAL_TFLOPS = 1.25


# ---------------------------------------------------------- CPU baseline
def cpu_sample_seconds_per_q(w, nk_sample=2, nom_sample=8, threads=0):
    """The reference's CPU path restated (oracle), timed on a bounded sample:
    the weights for ``nom_sample`` of the frequencies (the work is linear in
    them), the contraction for ``nk_sample`` k-points at every frequency, and
    the inverse for ``nom_sample`` frequencies; each part is scaled to the full
    q-point.  Returns (seconds per q, description)."""
    from oracle import weights as ow
    from pygw_gb300 import synthetic as syn
    import scipy.linalg
    p = syn.Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    om = p.fr.omega
    osel = np.linspace(0, len(om) - 1, min(nom_sample, len(om))).round().astype(int)
    t0 = time.perf_counter()
    kcw_s = ow.bz_calcqdepw_par2(b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, om[osel], p.kqm.tetc,
                                 nthreads=threads)
    t_w = (time.perf_counter() - t0) * len(om) / len(osel)
    sqv = syn.coulomb_sqrt(w, iq, w.npb)
    nkp = p.kqm.nkp
    nb1, nb2 = kcw_s.shape[:2]
    ks = list(range(min(nk_sample, nkp)))
    mins = [syn.minm_k(w, b, p.kqm, iq, ik, sqv) for ik in ks]
    eps = np.zeros((w.npb, w.npb, len(om)), dtype=complex, order="F")
    t0 = time.perf_counter()
    for j, ik in enumerate(ks):                  # pygw.py:3170-3185
        minm2 = np.reshape(mins[j], (nb1 * nb2, w.npb))
        cminm2 = np.conj(minm2)
        minm2Tc = minm2.T * -2.0
        for iom in range(len(om)):
            tmat = minm2Tc * kcw_s[:, :, ik, iom % len(osel)].ravel()
            eps[:, :, iom] += np.matmul(tmat, cminm2)
    t_c = (time.perf_counter() - t0) * nkp / len(ks)
    t0 = time.perf_counter()
    Id = np.identity(w.npb)
    for iom in osel:                             # pygw.py:3231-3268
        e = (eps[:, :, iom] + np.conj(eps[:, :, iom].T)) / 2.0 + Id
        eps[:, :, iom] = scipy.linalg.inv(e) - Id
    t_i = (time.perf_counter() - t0) * len(om) / len(osel)
    desc = (f"oracle C++ weights on {len(osel)}/{len(om)} frequencies ({os.cpu_count()} threads) scaled: {t_w:.2f}s; "
            f"numpy contraction on {len(ks)}/{nkp} k-points, all frequencies, scaled: {t_c:.2f}s; numpy inverse "
            f"on {len(osel)}/{len(om)} frequencies scaled: {t_i:.2f}s")
    measured = {"weights": len(osel) / len(om), "contraction": len(ks) / nkp, "inverse": len(osel) / len(om)}
    return t_w + t_c + t_i, desc, measured


def run_reference(a, w, rank):
    if rank != 0:
        return
    from oracle.build import build as build_oracle
    build_oracle()
    cpu_sample_seconds_per_q(w, nk_sample=2)      # warm caches/threads (outside timing)
    times, desc, measured = [], "", {}
    for i in range(a.warmup + a.steps):
        t, desc, measured = cpu_sample_seconds_per_q(w)
        if i >= a.warmup:
            times.append(t)
    v = max(times)
    line = {"metric": "s/q-point for chi0+eps^-1 (weights -> chi0 -> eps^-1)", "value": v, "unit": "s/q-point",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_desc(w), "precision": "fp64", "parallelism": "replicas"},
            "cpu_baseline": {"value": v, "unit": "s/q-point", "cores": os.cpu_count(), "kind": "port",
                             "sample": desc, "extrapolated": True, "measured_fraction": measured},
            "extrapolated": True,
            "extrapolation": ("each step times a bounded sample of the q-point (fractions in "
                              "cpu_baseline.measured_fraction, each part linear in what it samples) and scales it to "
                              "the whole q-point, so value and ms_per_step are modelled, not a wall-clock step"),
            "e2e": {"value": v, "unit": "s/q-point", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- batched workload
def run_batch_workload(a, w, rank, world, sampler):
    """C4 (q points of uneven N_PB and ragged per-k windows) and C5 (matrix
    elements too large to hold: drawn per k-chunk on the device; q = Γ with
    head and wings) through the batch driver, one captured CUDA graph per step
    unless --no-graph; value = step time / q points of the step."""
    import torch
    from pygw_gb300 import _lib
    from pygw_gb300 import batch as pb
    from pygw_gb300 import eps as peps
    from pygw_gb300 import synthetic as syn
    from pygw_gb300.device import ptr, stream_handle
    lib = _lib.load()
    prob = syn.Problem(w)
    tasks = (pb.c5_tasks(prob) if not w.npb_range else pb.c4_tasks(prob))
    if a.q_limit:
        tasks = tasks[:a.q_limit]
    from pygw_gb300 import replicas
    tasks = replicas.my_points(tasks, rank, world) or tasks[:1]
    t0 = time.time()
    tuner = None if a.no_tune else pb.Tuner(path=a.tune_file)
    bt = pb.batch_for(prob, tasks, tuner=tuner)
    graph = not a.no_graph
    if graph:
        bt.capture()
    setup_s = time.time() - t0
    stream = torch.cuda.current_stream()
    l0 = lib.pg_launch_count()
    for _ in range(a.warmup):
        bt.run(graph=graph)
    torch.cuda.synchronize()
    per_run = bt.graph_launches if graph else (lib.pg_launch_count() - l0) // max(1, a.warmup)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    wall0 = time.time()
    ev0.record(stream)
    for _ in range(a.steps):
        bt.run(graph=graph)
    ev1.record(stream)
    torch.cuda.synchronize()
    wall1 = time.time()
    dt = ev0.elapsed_time(ev1) * 1e-3
    status = bt.status()
    nq = len(tasks)
    value = dt / (a.steps * nq)
    nb1, nb2, nkp, nom = bt.nb1, bt.nb2, bt.nkp, bt.nom
    alg = sum(8.0 * t.npb * t.npb * k * nom for t, k in zip(tasks, bt.ktot))   # ragged K = Σ_k nb1·knb2[k]
    peak, peak_note = bf16_peak()
    roof = {"kernel": "whole step (weights + split-precision chi0 + mixed eps^-1, one graph)", "bound": "tensor",
            "achieved": alg / (dt / a.steps) / 1e12, "peak": peak, "unit": "TFLOP/s",
            "frac": alg / (dt / a.steps) / 1e12 / peak, "traffic": None,
            "note": "algorithmic 8*N_q^2*K_q*Nw summed over q (K_q = ragged window total) / step time; "
                    "the per-kernel roofline of k_ozaki_gemm is in the C3 line; peak = bf16 " + peak_note}
    # plain FP64 GPU path, one q at a time on the full window: weights and inverse timed in full,
    # the FP64 contraction on a few k-points (device-generated M) and scaled
    fp64 = None
    if a.fp64_k_sample > 0:
        tot, parts = 0.0, []
        sample = tasks[:: max(1, len(tasks) // 3)][:3]
        for t in sample:
            i = tasks.index(t)
            nk = min(a.fp64_k_sample, nkp)
            m = torch.empty((nk * nb1 * nb2, t.npb), dtype=torch.complex128, device="cuda")
            _lib.check(lib.pg_synth_minm(nk, 0, t.iq, ptr(bt.enk_d), bt.nbnd, ptr(bt.kqid_d[t.iq]), bt.ncg, bt.numin,
                                         nb1, nb2, None, None, 0, ptr(bt.sqv_d[i]), t.npb, bt.seed, ptr(m),
                                         stream_handle(None)), "pg_synth_minm")
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record()
            bt._weights(i, stream_handle(None))
            ev[1].record()
            eps = torch.zeros((nom, t.npb, t.npb), dtype=torch.complex128, device="cuda")
            _lib.check(lib.pg_chi0_accumulate_f64(ptr(m), nk, 0, ptr(bt.kcw), nb1, nb2, nkp, nom, t.npb, -2.0,
                                                  ptr(eps), None, None, stream_handle(None)), "pg_chi0_accumulate_f64")
            peps.chi0_finalize(eps, t.npb, nom)
            ev[2].record()
            peps.eps_inverse(eps, t.npb, nom, precision="fp64")
            ev[3].record()
            torch.cuda.synchronize()
            sq = (ev[0].elapsed_time(ev[1]) + ev[1].elapsed_time(ev[2]) * nkp / nk + ev[2].elapsed_time(ev[3])) * 1e-3
            parts.append({"npb": t.npb, "s": sq})
            tot += sq
            del m, eps
        fp64 = {"value": tot / len(sample), "unit": "s/q-point", "per_q": parts,
                "sample": f"{len(sample)} of {nq} q; FP64 contraction on {min(a.fp64_k_sample, nkp)}/{nkp} "
                          f"k-points of the full window, scaled"}
    # end to end: host inputs of the batch to the device, the graph, every q's eps^-1 back to pinned host memory
    e2e = None
    if not a.no_e2e:
        outs = [torch.empty(r.shape, dtype=r.dtype).pin_memory() for r in bt.results]
        b = prob.bands
        nomx, numin = b.nomax_numin
        host_in = [torch.from_numpy(np.ascontiguousarray(b.enk().T)).pin_memory(),
                   torch.from_numpy(np.ascontiguousarray(prob.kqm.tetc.T.astype(np.int32))).pin_memory(),
                   torch.from_numpy(prob.fr.omega.copy()).pin_memory()]
        torch.cuda.synchronize()
        te0 = time.perf_counter()
        for _ in range(a.steps):
            bt.enk_d.copy_(host_in[0], non_blocking=True)
            bt.tetc_d.copy_(host_in[1], non_blocking=True)
            bt.om_d.copy_(host_in[2], non_blocking=True)
            bt.run(graph=graph)
            for o, r in zip(outs, bt.results):
                o.copy_(r, non_blocking=True)
        torch.cuda.synchronize()
        et = time.perf_counter() - te0
        e2e = {"value": et / (a.steps * nq), "unit": "s/q-point",
               "h2d_bytes_per_step": int(sum(x.numel() * x.element_size() for x in host_in)),
               "d2h_bytes_per_step": int(sum(o.numel() * 16 for o in outs))}
    sampler.stop()
    clocks = sampler.window(wall0, wall1)
    sampler.cleanup()
    if rank == 0:
        line = {"metric": "s/q-point for chi0+eps^-1 (weights -> chi0 -> eps^-1)", "value": value,
                "unit": "s/q-point", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
                "ms_per_step": dt / a.steps * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16-digits/f32-exact/f64", "data": "synthetic",
                "config": {"workload": workload_desc(w) + f", N_PB per q {[t.npb for t in tasks]}"
                                                          + (", per-k unoccupied cutoff 100-300 bands" if w.npb_range
                                                             else f", q {[t.iq for t in tasks]} (q=0: head and "
                                                                  f"wings)"),
                           "precision": "mixed", "parallelism": "replicas",
                           "batch": {"q_per_step": nq, "graph": graph, "setup_s": setup_s,
                                     "tuned": [[c.k_chunk, c.omega_batch] for c in bt.choice]},
                           "l2": "inputs larger than L2 (matrix elements drawn per k-chunk on the device)"},
                "roofline": roof, "kernel_status": status, "fp64_gpu": fp64, "cpu_baseline": None,
                "e2e": e2e, "gpu_launches": int(per_run * a.steps), "clocks": clocks}
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------- self-energy
def run_selfc(a, w, rank, world, sampler):
    """Seconds per q-point of calc_selfc's GPU body (pygw.py:3335-3385): mwm
    over every k-point (split precision, or FP64 with --precision fp64) and the
    Matsubara convolution (all_fr_convolutions).  nb1 = --selfc-nb1 GW bands,
    nb2 = all bands of the workload, M drawn on the device and resident, ε⁻¹−1
    a seeded negative semidefinite Hermitian matrix per frequency."""
    import torch
    from pygw_gb300 import _lib
    from pygw_gb300 import selfc as gsc
    from pygw_gb300 import synthetic as syn
    from pygw_gb300.device import ptr, stream_handle
    lib = _lib.load()
    prob = syn.Problem(w)
    b = prob.bands
    kqm = prob.kqm
    nkp, N, nom = kqm.nkp, w.npb, w.nom
    enk = b.enk()                                     # [nbnd, nkp]
    nbnd = enk.shape[0]
    nb1, nb2 = min(a.selfc_nb1, nbnd), nbnd
    P = nb1 * nb2
    from pygw_gb300 import replicas
    qs = replicas.my_points(list(prob.qs), rank, world) or list(prob.qs[:1])
    iq = qs[0]
    enk_d = torch.from_numpy(np.ascontiguousarray(enk.T)).cuda()
    kq_d = torch.from_numpy(np.ascontiguousarray(kqm.kqid[:, iq].astype(np.int32))).cuda()
    sqv_d = torch.from_numpy(syn.coulomb_sqrt(w, iq, N)).cuda()
    M = torch.empty((nkp, P, N), dtype=torch.complex128, device="cuda")
    _lib.check(lib.pg_synth_minm(nkp, 0, iq, ptr(enk_d), nbnd, ptr(kq_d), 0, 0, nb1, nb2, None, None, 0, ptr(sqv_d),
                                 N, w.seed, ptr(M), stream_handle(None)), "pg_synth_minm")
    g = torch.Generator(device="cuda").manual_seed(w.seed)
    W = torch.empty((nom, N, N), dtype=torch.complex128, device="cuda")
    for iw in range(nom):                             # ε⁻¹ − 1 ≤ 0, decaying with the frequency
        B = torch.randn((N, N), dtype=torch.complex128, device="cuda", generator=g)
        W[iw] = -(B @ B.conj().T) * (0.5 / N / (1.0 + prob.fr.omega[iw]))
    # k-points at k−q in the energy list of the convolution (no core states here)
    ekq = np.stack([enk[:, int(kqm.kqid[ik, iq])] for ik in range(nkp)])          # [nkp][nb2]
    om = prob.fr.omega
    wom = np.gradient(om)
    wkq = 1.0 / nkp
    precision = a.precision
    budget = 24 << 30
    k_chunk, nb = gsc.mixed_k_chunk(P, N, nom, budget) if precision == "mixed" else (nkp, nom)
    k_chunk = min(k_chunk, nkp)
    workspace_mixed = None
    if precision == "mixed":
        workspace_mixed = torch.empty(lib.pg_selfc_mwm_workspace(k_chunk, P, N, nb, 1), dtype=torch.uint8,
                                      device="cuda")
    mwm_d = torch.empty((nkp, nom, P), dtype=torch.complex128, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    om_d = torch.from_numpy(om.copy()).cuda()
    wom_d = torch.from_numpy(wom).cuda()
    ekq_d = torch.from_numpy(ekq).cuda()
    sc_d = torch.empty((nkp, nb1, nom), dtype=torch.complex128, device="cuda")
    stream = torch.cuda.current_stream()
    sh = stream_handle(None)
    g_ev = []

    def step(timed=False, phases=None):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)] if phases is not None else None
        if ev:
            ev[0].record(stream)
        for k0 in range(0, nkp, k_chunk):
            nk = min(k_chunk, nkp - k0)
            if timed:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            rc = lib.pg_selfc_mwm(ptr(M[k0]), nk, P, N, ptr(W), nom, wkq, ptr(mwm_d[k0]),
                                  1 if precision == "mixed" else 0, nb, ptr(workspace_mixed),
                                  0 if workspace_mixed is None else workspace_mixed.numel(), ptr(status), sh)
            _lib.check(rc, "pg_selfc_mwm")
            if timed:
                e1.record(stream)
                g_ev.append((e0, e1, nk))
        if ev:
            ev[1].record(stream)
        rc = lib.pg_selfc_convolution(ptr(mwm_d), nkp, nb1, nb2, nom, ptr(ekq_d), ptr(om_d), ptr(wom_d), 0, None,
                                      None, None, None, 0, ptr(sc_d), sh)
        _lib.check(rc, "pg_selfc_convolution")
        if ev:
            ev[2].record(stream)
            phases.append(ev)

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    phases = []
    l0 = lib.pg_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    wall0 = time.time()
    ev0.record(stream)
    for _ in range(a.steps):
        step(timed=True, phases=phases)
    ev1.record(stream)
    torch.cuda.synchronize()
    wall1 = time.time()
    launches = lib.pg_launch_count() - l0
    dt = ev0.elapsed_time(ev1) * 1e-3
    value = dt / a.steps
    phase_ms = {name: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in phases)
                for i, name in enumerate(["mwm", "convolution"])}
    # roofline of the contraction: the reference's complex GEMM count 8·P·N²·nω per k-point
    mw_s = sum(e0.elapsed_time(e1) for e0, e1, _ in g_ev) * 1e-3
    alg = sum(8.0 * nk * P * N * N * nom for _, _, nk in g_ev)
    if precision == "mixed":
        peak, note = bf16_peak()
        rpad_b = -(-N // 256) * 256
        kpad = -(-2 * N // 64) * 64
        exe = sum(15 * 2.0 * (-(-2 * nk * P // 256) * 256) * min(rpad_b, -(-N // 128) * 128) * kpad * nom
                  for _, _, nk in g_ev)
        roof = {"kernel": "pg_selfc_mwm (k_rows_digits + per frequency batch: column digits, k_ozaki_gemm general "
                          "mode, k_mwm_reduce)", "bound": "tensor", "achieved": alg / mw_s / 1e12, "peak": peak,
                "unit": "TFLOP/s", "frac": alg / mw_s / 1e12 / peak, "traffic": None,
                "executed_bf16_tflops": exe / mw_s / 1e12, "executed_frac": exe / mw_s / 1e12 / peak,
                "note": "achieved = 8*P*N^2*Nw per k (the reference's complex matmul count) / CUDA-event time of "
                        "the contraction calls; executed = 15 digit-pair bf16 products of the (2R x 2N)(2N x N) "
                        "real form; peak = bf16 " + note}
    else:
        peak = FP64_NOMINAL_TFLOPS
        roof = {"kernel": "k_mwm_f64", "bound": "fp64", "achieved": alg / mw_s / 1e12, "peak": peak,
                "unit": "TFLOP/s", "frac": alg / mw_s / 1e12 / peak, "traffic": None,
                "note": "peak = nominal GB300 FP64 (no measured FP64 figure available)"}
    # the plain FP64 GPU contraction on a few k-points, scaled
    fp64 = None
    if precision == "mixed" and a.fp64_k_sample > 0:
        nk = min(a.fp64_k_sample, nkp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(lib.pg_selfc_mwm(ptr(M), nk, P, N, ptr(W), nom, wkq, ptr(mwm_d), 0, nom, None, 0, ptr(status),
                                    sh), "pg_selfc_mwm")
        e1.record(stream)
        torch.cuda.synchronize()
        t_m = e0.elapsed_time(e1) * 1e-3 * nkp / nk
        fp64 = {"value": t_m + phase_ms["convolution"] * 1e-3, "unit": "s/q-point", "mwm_s": t_m,
                "sample": f"FP64 contraction timed on {nk}/{nkp} k-points and scaled; convolution as measured"}
    # end to end through the Python API: M from pinned host memory per k-chunk, Σc back to the host
    e2e = None
    if not a.no_e2e:
        M_h = torch.empty((nkp, P, N), dtype=torch.complex128).pin_memory()
        M_h.copy_(M)
        sc_h = torch.empty((nkp, nb1, nom), dtype=torch.complex128).pin_memory()
        ch = k_chunk if precision == "mixed" else max(1, min(nkp, int((4 << 30) // (16 * P * N))))

        def e2e_step():
            out = torch.empty((nkp, nom, P), dtype=torch.complex128, device="cuda")
            for k0 in range(0, nkp, ch):
                k1 = min(nkp, k0 + ch)
                gsc.mwm(M_h[k0:k1], W, nb1, nb2, wkq, precision=precision, omega_batch=nb, out=out[k0:k1],
                        work=workspace_mixed, status=status)
            sc = gsc.convolution(out, ekq, om, wom, nb1, nb2)
            sc_h.copy_(sc)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e2e_step()
        torch.cuda.synchronize()
        et = time.perf_counter() - t0
        e2e = {"value": et / a.steps, "unit": "s/q-point", "h2d_bytes_per_step": int(M_h.numel() * 16),
               "d2h_bytes_per_step": int(sc_h.numel() * 16)}
        del M_h
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        from oracle import selfc as osc
        Mh = M[0].cpu().numpy().reshape(nb1, nb2, N)
        Wh = W.cpu().numpy().transpose(2, 1, 0)                # (N, N, nom)
        t0 = time.perf_counter()
        mw = osc.mwm_k(Mh, Wh, wkq)
        t_m = (time.perf_counter() - t0) * nkp
        rows = 2
        t0 = time.perf_counter()
        osc.all_fr_convolutions(ekq[0], mw[:, :rows, :], om, wom)
        t_c = (time.perf_counter() - t0) * nkp * nb1 / rows
        cpu = {"value": t_m + t_c, "unit": "s/q-point", "cores": os.cpu_count(), "kind": "port",
               "sample": f"numpy mwm (pygw.py:3352-3356) on 1/{nkp} k-points, all {nom} frequencies, scaled: "
                         f"{t_m:.1f}s; the restated convolution (fnc.f90:90-177, Python loops) on {rows}/{nb1} "
                         f"bands of 1 k-point, scaled: {t_c:.1f}s"}
    st = int(status.item())
    sampler.stop()
    clocks = sampler.window(wall0, wall1)
    sampler.cleanup()
    if rank == 0:
        line = {"metric": "s/q-point for calc_selfc's mwm contraction + Matsubara convolution", "value": value,
                "unit": "s/q-point", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
                "ms_per_step": dt / a.steps * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "bf16-digits/f32-exact/f64",
                "data": "synthetic",
                "config": {"workload": workload_desc(w) + f"; selfc: nb1 {nb1} GW bands x nb2 {nb2} bands, "
                                                          f"P {P}, {nkp} k-points, q {iq}",
                           "precision": precision, "parallelism": "replicas", "k_chunk": k_chunk,
                           "omega_batch": nb,
                           "l2": "inputs larger than L2 (matrix elements %.1f GB read every step)"
                                 % (M.numel() * 16 / 1e9)},
                "roofline": roof, "kernel_status": st, "phases_ms": phase_ms, "fp64_gpu": fp64,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks}
        print(json.dumps(line), flush=True)


# -------------------------------------------------------------------- main
def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    from pygw_gb300.synthetic import WORKLOADS, scaled
    w = WORKLOADS[a.workload]
    if a.div or a.npb or a.nom:
        w = scaled(w, div=a.div or w.div, npb=a.npb or w.npb, nom=a.nom or w.nom)
    if a.impl == "reference":
        return run_reference(a, w, rank)

    local = int(os.environ.get("LOCAL_RANK", "0"))
    sampler = ClockSampler(local)
    sampler.start()                    # before CUDA is initialised in this process
    import __graft_entry__
    __graft_entry__.build()            # any compiler subprocess also runs before CUDA init
    from oracle.build import build as build_oracle
    build_oracle()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pygw_gb300 import _lib
    _lib.check(_lib.load().pg_set_chi0_prep_batch(a.prep_batch), "pg_set_chi0_prep_batch")

    if a.path == "selfc":
        return run_selfc(a, w, rank, world, sampler)
    if w.npb_range or w.name == "C5":
        return run_batch_workload(a, w, rank, world, sampler)
    lib = _lib.load()
    inp = Inputs(w, rank)
    inp.statuses = []
    inp.gemm_timers = []
    if a.precision == "mixed":
        from pygw_gb300 import eps as peps
        inp.wb = a.omega_batch or peps.mixed_omega_batch(inp.nb1, inp.nb2, inp.nkp, w.npb, w.nom)
    inp.kb_split = a.kb_split
    # replicas: each rank runs its contiguous block of q points (the reference's mpiSplitArray)
    from pygw_gb300 import replicas
    inp.qs = replicas.my_points(inp.qs, rank, world) or inp.qs[:1]

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    for s in range(a.warmup):
        gpu_step(inp, s, precision=a.precision)
    barrier()
    timers = []
    phases = []
    l0 = lib.pg_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    wall0 = time.time()
    ev0.record(stream)
    for s in range(a.steps):
        gpu_step(inp, a.warmup + s, timers=timers, precision=a.precision, phases=phases)
    ev1.record(stream)
    barrier()
    wall1 = time.time()
    launches = lib.pg_launch_count() - l0
    dt = ev0.elapsed_time(ev1) * 1e-3
    if dist is not None:
        t = torch.tensor([dt], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
    value = dt / (a.steps * world)               # seconds per q-point, whole job
    # dominant kernel: the χ0 contraction (one launch sequence per step)
    chi0_ms = [s_.elapsed_time(e_) for s_, e_ in timers]
    nb1, nb2, npb, nom = inp.nb1, inp.nb2, w.npb, w.nom
    flops = 8.0 * npb * npb * nb1 * nb2 * inp.nkp * nom     # full complex GEMM count (reference's ZGEMMs)
    achieved = flops / (statistics.mean(chi0_ms) * 1e-3) / 1e12
    status_bits = 0
    for st in inp.statuses:
        status_bits |= int(st.item())
    if a.precision == "mixed":
        peak, peak_note = bf16_peak()
        kpad = ((inp.nkp * nb1 * nb2 + 63) // 64) * 64
        # per launch: one batch of wb frequencies (the last batch may be smaller)
        g_ms = [s_.elapsed_time(e_) for s_, e_ in inp.gemm_timers]
        nbatch = -(-nom // inp.wb)
        nws = [min(inp.wb, nom - b * inp.wb) for b in range(nbatch)] * (len(g_ms) // nbatch)
        alg = sum(8.0 * npb * npb * nb1 * nb2 * inp.nkp * nw for nw in nws)
        exe = sum(15 * 2.0 * mixed_tile_area(npb) * kpad * nw for nw in nws)
        g_s = sum(g_ms) * 1e-3
        # distinct digit bytes of one launch: the A planes once, the B planes of each frequency
        rpad = -(-2 * npb // 256) * 256
        dig_bytes = 5 * rpad * kpad * 2 * (1 + inp.wb)
        tkey = (GEMM_BUILD, w.name, npb, inp.nkp, inp.wb)
        traffic, traffic_src = MEASURED_GEMM_TRAFFIC.get(tkey, (None, None))
        hbm = json.load(open(PEAKS_FILE)).get("hbm_gbs") if os.path.exists(PEAKS_FILE) else None
        roof = {"kernel": "k_ozaki_gemm", "bound": "tensor", "achieved": alg / g_s / 1e12,
                "peak": peak, "unit": "TFLOP/s", "frac": alg / g_s / 1e12 / peak, "traffic": traffic,
                "traffic_source": traffic_src or f"no ncu capture of this kernel build at this launch shape {tkey}",
                "algorithmic_bytes": dig_bytes,
                "dram_frac": (traffic / (g_s / len(g_ms)) / 1e9 / hbm) if traffic and hbm else None,
                "launches": len(g_ms), "ms_per_launch": sum(g_ms) / max(1, len(g_ms)),
                "executed_bf16_tflops": exe / g_s / 1e12,
                "executed_frac": exe / g_s / 1e12 / peak,
                "chi0_phase_algorithmic_tflops": achieved,
                "note": "achieved = 8*N_PB^2*P*Nk*Nw per launch (the reference's complex FP64 GEMM count) / "
                        "CUDA-event launch time of k_ozaki_gemm; executed_bf16 = 15 digit-pair bf16 products "
                        "over the computed 256x256 blocks; peak = bf16 " + peak_note + "; traffic = "
                        "DRAM bytes per launch from one ncu capture of this kernel build and launch shape "
                        "(traffic_source; null if not captured), "
                        "algorithmic_bytes = the distinct digit planes the launch reads, dram_frac = traffic / "
                        "launch time / measured HBM copy bandwidth"}
    else:
        peak = FP64_NOMINAL_TFLOPS
        roof = {"kernel": "k_chi0_f64", "bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None,
                "note": "algorithmic flops = 8*N_PB^2*P*Nk*Nw (full complex GEMM count) per launch; "
                        "peak = nominal GB300 FP64 (no measured FP64 figure available)"}

    phase_ms = {name: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in phases)
                for i, name in enumerate(["weights", "chi0", "eps_inverse"])}
    fp64 = None
    if a.precision == "mixed" and a.fp64_k_sample > 0:
        v64, parts = fp64_gpu_estimate(inp, a.fp64_k_sample)
        fp64 = {"value": v64, "unit": "s/q-point", **parts}
    roof_w = weights_roofline(inp)
    acc = None
    if a.precision == "mixed" and not a.no_accuracy:
        acc = measure_accuracy(inp)

    e2e = None
    if not a.no_e2e:
        # the public-API run starts from the state a caller has: the device
        # copies and workspace of the resident measurement are released first
        inp.minm_dev = None
        inp.mwork = None
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        out_host = inp.out_h
        for s in range(min(a.warmup, 1)):
            e2e_step(inp, s, out_host, a.precision)
        barrier()
        t0 = time.perf_counter()
        for s in range(a.steps):
            e2e_step(inp, s, out_host, a.precision)
        torch.cuda.synchronize()
        et = time.perf_counter() - t0
        if dist is not None:
            t = torch.tensor([et], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            et = float(t.item())
        h2d = (inp.minm_host.numel() * 16 + inp.enk.nbytes + inp.tetc.nbytes // 2 + inp.nkp * 4
               + inp.omega.nbytes)
        e2e = {"value": et / (a.steps * world), "unit": "s/q-point", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(out_host.numel() * 16)}

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        v, desc, measured = cpu_sample_seconds_per_q(w)
        cpu = {"value": v, "unit": "s/q-point", "cores": os.cpu_count(), "kind": "port", "sample": desc,
               "extrapolated": True, "measured_fraction": measured}

    torch.cuda.synchronize()
    sampler.stop()
    clocks = sampler.window(wall0, wall1)
    sampler.cleanup()
    if rank == 0:
        line = {"metric": "s/q-point for chi0+eps^-1 (weights -> chi0 -> eps^-1)", "value": value,
                "unit": "s/q-point", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
                "ms_per_step": dt / a.steps * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if a.precision == "fp64" else "bf16-digits/f32-exact/f64",
                "data": "synthetic",
                "config": {"workload": workload_desc(w), "precision": a.precision, "parallelism": "replicas",
                           "chi0_prep_batch": lib.pg_chi0_prep_batch() if a.precision == "mixed" else None,
                           "l2": "inputs larger than L2 (matrix elements %.2f GB read every step)"
                                 % (inp.minm_host.numel() * 16 / 1e9)},
                "roofline": roof, "roofline_weights": roof_w, "accuracy": acc, "kernel_status": status_bits,
                "phases_ms": phase_ms, "fp64_gpu": fp64, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": int(launches), "clocks": clocks}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
