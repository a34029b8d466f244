"""The allocation-free weight entry point, through the C-ABI (GPU).

pg_bz_calcqdepw_par2_noalloc serves callers that cannot allocate device
memory — host programs reaching the library through a foreign-function layer
with no device allocator of their own, or services held to a fixed memory
budget.  Its scratch is a fixed device array inside the library.  This test
calls it twice in a row (the second call finds the first call's contents in
that array) and compares each result with the regular entry point, which the
caller gives a workspace.  The weights are computed by the same kernels in
the same order, so the comparison is exact (tolerance 0).  It also checks
that a problem too large for the array is rejected.

This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest
import torch

from pygw_gb300 import _lib
from pygw_gb300 import polarization as pol
from pygw_gb300.synthetic import WORKLOADS, Problem, scaled

pytestmark = pytest.mark.gpu


def _inputs(w):
    p = Problem(w)
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0]
    enk = torch.from_numpy(np.ascontiguousarray(b.enk().T)).cuda()                      # [nkp][nbnd]
    tetc = torch.from_numpy(np.ascontiguousarray(p.kqm.tetc.T.astype(np.int32))).cuda()  # [ntet][4]
    kqid = torch.from_numpy(np.ascontiguousarray(p.kqm.kqid[:, iq].astype(np.int32))).cuda()
    om = torch.from_numpy(p.fr.omega.copy()).cuda()
    return p, b, nomx, numin, enk, tetc, kqid, om


def _noalloc(lib, b, nomx, numin, enk, tetc, kqid, om, kcw, status, counters):
    nkp, nbnd = enk.shape
    return lib.pg_bz_calcqdepw_par2_noalloc(enk.data_ptr(), nbnd, nkp, float(b.EF), kqid.data_ptr(), 0, nomx, numin,
                                            om.data_ptr(), om.shape[0], tetc.data_ptr(), tetc.shape[0],
                                            kcw.data_ptr(), status.data_ptr(), counters.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("name", ["C1", "C2"])
def test_noalloc_matches_regular_entry_point_twice(name):
    lib = _lib.load()
    p, b, nomx, numin, enk, tetc, kqid, om = _inputs(WORKLOADS[name])
    ref = pol.weights_device(enk, b.EF, kqid, 0, nomx, numin, om, tetc)
    torch.cuda.synchronize()
    ref_kcw = ref.kcw.cpu().numpy()
    for call in range(2):
        kcw = torch.full_like(ref.kcw, np.nan)
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        counters = torch.zeros(len(pol.STAT_NAMES), dtype=torch.int64, device="cuda")
        rc = _noalloc(lib, b, nomx, numin, enk, tetc, kqid, om, kcw, status, counters)
        assert rc == 0, f"call {call}: {_lib.ERRORS.get(rc, rc)}"
        torch.cuda.synchronize()
        got = kcw.cpu().numpy()
        assert np.max(np.abs(got - ref_kcw)) <= 0.0, f"call {call}"
        assert int(status.item()) == ref.status
        # per-(sub-tetrahedron, ω) counters are chunk-independent; the geometry
        # counters are counted once per frequency chunk
        got_c = dict(zip(pol.STAT_NAMES, counters.cpu().tolist()))
        for k in ("taylor", "exact", "big_weight_warn", "big_weight_zeroed"):
            assert got_c[k] == ref.counters[k], k
        assert got_c["calls"] % ref.counters["calls"] == 0


def test_noalloc_rejects_problems_beyond_its_array():
    lib = _lib.load()
    cap = lib.pg_bz_calcqdepw_par2_noalloc_capacity()
    assert cap == 256 << 20
    # 10^3 mesh, 39 x 376 band pairs: one frequency of scratch is 2.8 GB > the array.
    w = scaled(WORKLOADS["C5"], nom=2)
    p, b, nomx, numin, enk, tetc, kqid, om = _inputs(w)
    kcw = torch.empty(1, dtype=torch.float64, device="cuda")      # never touched: rejected before any launch
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    counters = torch.zeros(len(pol.STAT_NAMES), dtype=torch.int64, device="cuda")
    rc = _noalloc(lib, b, nomx, numin, enk, tetc, kqid, om, kcw, status, counters)
    assert rc == -4
