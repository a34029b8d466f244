"""How close the split-precision ε⁻¹ is to the plain FP64 one, on chosen frequencies.

A diagnostic for callers (and the benchmark): the same weights and matrix
elements go through both GPU paths — the FP64 contraction and Gauss–Jordan
inverse, and the split-precision tensor-core contraction with the FP32
inverse refined in FP64 — for a few frequencies, and the two ε⁻¹ are compared
(pygw.py:3229-3271 is the reference's inverse).  Two figures per frequency:

* normwise: max |Δ| / max |ε⁻¹_ref|, the bar the split-precision path is held to
  (1e-9);
* element-wise: max |Δ_ij| / |ε⁻¹_ref,ij| over the entries with |ε⁻¹_ref,ij|
  above ``floor`` · max |ε⁻¹_ref| (smaller entries carry no relative digits
  worth quoting: their absolute error is bounded by the normwise figure).

The FP64 contraction costs about 5 s per frequency at N_PB = 1200 with 216
k-points; pick few frequencies.
"""
from __future__ import annotations

import torch

from . import eps as peps


def mixed_vs_fp64(kcw_d, minm, nkp, npb, nb1, nb2, freqs, floor=1e-8, floors=(1e-6, 1e-4, 1e-2)):
    """``kcw_d``: device weights [nom][nkp][nb2][nb1] (the weights kernel's
    layout); ``minm``: [nkp, nb1·nb2, npb] complex128 on the device (or any
    source ``eps.chi0_accumulate`` takes); ``freqs``: frequency indices.
    Returns a dict of per-frequency and worst errors; ``elementwise_by_floor``
    gives the worst element-wise error over the entries above each of
    ``floors`` too (how the error spreads from large to small entries)."""
    freqs = [int(f) for f in freqs]
    sel = kcw_d[freqs].contiguous()
    n = len(freqs)
    ref = peps.chi0_eps(sel, minm, nkp, npb, nb1, nb2, n, precision="fp64")
    got = peps.chi0_eps(sel, minm, nkp, npb, nb1, nb2, n, precision="mixed")
    torch.cuda.synchronize()
    status = int(got.chi0_status.item()) | int(got.status.item())
    eye = torch.eye(npb, dtype=torch.complex128, device=sel.device)
    normwise, elementwise, diag = [], [], []
    by_floor = {f"{f:g}": 0.0 for f in floors}
    for i in range(n):
        r = ref.eps[i] + eye
        g = got.eps[i] + eye
        d = (g - r).abs()
        ra = r.abs()
        mx = ra.max()
        normwise.append(float(d.max() / mx))
        mask = ra > floor * mx
        rel = d / ra.clamp_min(1e-300)
        elementwise.append(float(rel[mask].max()))
        for f in floors:
            by_floor[f"{f:g}"] = max(by_floor[f"{f:g}"], float(rel[ra > f * mx].max()))
        diag.append(float((d.diagonal() / ra.diagonal()).max()))
    return {"frequencies": freqs, "normwise": normwise, "elementwise": elementwise, "diagonal": diag,
            "max_normwise": max(normwise), "max_elementwise": max(elementwise), "elementwise_floor": floor,
            "elementwise_by_floor": by_floor,
            "status": status}
