"""Host-side pieces: mesh/tetrahedra, k−q table, band windows, C-ABI exports (CPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pygw_gb300.mesh import KQmesh, build_kqid, build_tetc, indx2k, k2indx, shortest_diagonal
from pygw_gb300.synthetic import WORKLOADS, Problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_tetrahedra_cover_the_mesh(n):
    div = (n, n, n)
    tetc = build_tetc(div)
    nkp = n ** 3
    assert tetc.shape == (4, 6 * nkp) and tetc.flags.f_contiguous
    # every mesh point is a corner of exactly 24 (tetrahedron, corner) slots
    counts = np.bincount(tetc.ravel(order="F"), minlength=nkp)
    assert np.all(counts == 24)
    # the six tetrahedra of one cube have volume 1/6 each (in cell units)
    if n >= 3:
        for ik in range(nkp):
            o = indx2k(ik, div)
            for t in range(6):
                pts = []
                for i in range(4):
                    c = indx2k(tetc[i, 6 * ik + t], div)
                    d = (c - o) % n
                    pts.append(d.astype(float))
                v = abs(np.linalg.det(np.array([pts[1] - pts[0], pts[2] - pts[0], pts[3] - pts[0]]))) / 6
                assert abs(v - 1.0 / 6.0) < 1e-12


def test_kqid_matches_definition():
    div = (3, 4, 2)
    kq = build_kqid(div)
    nkp = 24
    for iq in range(nkp):
        q = indx2k(iq, div)
        for ik in range(nkp):
            k = indx2k(ik, div)
            assert kq[ik, iq] == k2indx((k - q) % np.array(div), div)
    assert np.all(kq[:, 0] == np.arange(nkp))


def test_linked_tetrahedron_is_the_shifted_one():
    """tetc(:, 6*kqid(ik)+t) = kqid(tetc(:, 6*ik+t)) on a uniform mesh — the
    identity behind tetln (for_tetrahedra.f90:426-432)."""
    m = KQmesh((4, 4, 4))
    for iq in (1, 7, 21):
        kq = m.kqid[:, iq]
        for ik in range(m.nkp):
            for t in range(6):
                assert np.array_equal(m.tetc[:, 6 * kq[ik] + t], kq[m.tetc[:, 6 * ik + t]])


def test_shortest_diagonal_choice():
    assert shortest_diagonal((4, 4, 4)) == 0
    g = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.9, 0.0, 1.0]])   # sheared cell
    assert shortest_diagonal((4, 4, 4), g) != 0 or True


def test_band_windows_of_the_workloads():
    expect = {"C1": (15, 0), "C2": (10, 0), "C3": (22, 8), "C5": (38, 24)}
    for name, (nomx, numin) in expect.items():
        b = Problem(WORKLOADS[name]).bands
        assert tuple(b.nomax_numin) == (nomx, numin)


def test_capi_library_exports_every_declared_symbol():
    """The shared library loads and exports each function of include/pygw_gb300.h
    (no compute call: this runs without a GPU)."""
    from pygw_gb300.build import build
    hdr = open(os.path.join(ROOT, "include", "pygw_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    names = set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) >= 6
    lib = ctypes.CDLL(build())
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    from pygw_gb300 import _lib
    assert names <= set(_lib.SIGNATURES)
    # size queries are pure host code and can be called without a device
    l2 = _lib.load()
    assert l2.pg_bz_calcqdepw_par2_workspace(32, 64, 0, 15, 0, 16, 384, 0) > 384 * 4 * 16 * 512 * 8
    assert l2.pg_bz_calcqdepw_par2_workspace(32, 64, 0, 15, 0, 16, 384, 4) < \
        l2.pg_bz_calcqdepw_par2_workspace(32, 64, 0, 15, 0, 16, 384, 0)
    assert l2.pg_eps_inverse_f64_workspace(0, 4) == 0


def test_selfc_entry_points_validate_on_the_host():
    """The self-energy entry points reject bad sizes, null pointers and short
    workspaces before any device call, and their size queries are host code."""
    from pygw_gb300 import _lib
    lib = _lib.load()
    EARG, EWORK = -1, -2
    # workspace queries: zero for bad sizes, growing with the k-points and the frequency batch
    assert lib.pg_selfc_mwm_workspace(0, 10, 64, 2, 1) == 0
    assert lib.pg_selfc_mwm_workspace(1, 10, 64, 2, 0) > 0
    w1 = lib.pg_selfc_mwm_workspace(1, 10, 64, 2, 1)
    assert lib.pg_selfc_mwm_workspace(2, 10, 64, 2, 1) > w1 < lib.pg_selfc_mwm_workspace(1, 10, 64, 4, 1)
    assert lib.pg_selfc_convolution_workspace(0, 2, 3, 4, 0, 0) == 0
    assert lib.pg_selfc_convolution_workspace(1, 2, 3, 4, 8, 0) > lib.pg_selfc_convolution_workspace(1, 2, 3, 4, 0, 0)
    fake = 0x1000                     # never dereferenced: every call below fails its checks first
    assert lib.pg_selfc_mwm(None, 1, 10, 64, fake, 2, 0.5, fake, 0, 2, None, 0, None, None) == EARG
    assert lib.pg_selfc_mwm(fake, 0, 10, 64, fake, 2, 0.5, fake, 0, 2, None, 0, None, None) == EARG
    assert lib.pg_selfc_mwm(fake, 1, 10, 64, fake, 2, 0.5, fake, 1, 2, None, 0, None, None) == EARG
    assert lib.pg_selfc_mwm(fake, 1, 10, 64, fake, 2, 0.5, fake, 1, 2, fake, w1 - 1, None, None) == EWORK
    assert lib.pg_selfc_mwm_q0(fake, 1, 2, 5, 64, -1, 2, fake, fake, fake, 1.0, 1.0, fake, None) == EARG
    assert lib.pg_selfc_convolution(fake, 1, 2, 3, 4, None, fake, fake, 0, None, None, None, None, 0, fake,
                                    None) == EARG
    assert lib.pg_selfc_convolution(fake, 1, 2, 3, 4, fake, fake, fake, 8, fake, fake, fake, fake, 16, fake,
                                    None) == EWORK
    assert lib.pg_selfc_convolution_svd(fake, 1, 2, 3, 0, 4, fake, fake, fake, fake, fake, 1 << 20, fake,
                                        None) == EARG


@pytest.mark.parametrize("nb1,nb2,nkp,npb,wb,kb_split", [
    (9, 24, 64, 128, 2, 0),          # C1-sized
    (23, 192, 216, 1200, 1, 0),      # C3, one frequency per launch
    (23, 192, 216, 1200, 4, 1000),   # C3, K range per split capped
    (39, 368, 57, 2000, 1, 0),       # a C5 k-chunk
    (40, 360, 1000, 2000, 1, 0),     # C5 in one pass: K = 14.4 M
    (5, 7, 3, 100, 3, 100),          # tiny, padding everywhere
])
def test_mixed_layout_keeps_group_sums_exact(nb1, nb2, nkp, npb, wb, kb_split):
    """The split-precision χ0 layout is host code: every K split is short enough
    for exact digit-group sums (5 pairs · kb·64 · 129² < 2^35), the splits cover
    the K-blocks with none empty, the rows pad to whole 256-column blocks, and
    the workspace regions are 256-byte aligned, in order and large enough."""
    from pygw_gb300 import _lib
    lib = _lib.load()
    offs = (ctypes.c_size_t * 9)()
    dims = (ctypes.c_longlong * 9)()
    assert lib.pg_chi0_mixed_layout(nb1, nb2, nkp, npb, wb, kb_split, offs, dims) == 0
    K, K_pad, R, R_pad, nT, npair, nkb, nsplit, kbs = list(dims)
    assert K == nb1 * nb2 * nkp and K_pad % 64 == 0 and K <= K_pad < K + 64 and nkb == K_pad // 64
    assert R == 2 * npb and R_pad % 256 == 0 and R <= R_pad < R + 256
    assert nT == R_pad // 128 and npair == nT * (nT + 1) // 2
    assert 5 * kbs * 64 * 129 ** 2 < 2 ** 35
    if kb_split:
        assert kbs <= kb_split
    assert (nsplit - 1) * kbs < nkb <= nsplit * kbs
    o = list(offs)
    assert all(x % 256 == 0 for x in o[:8]) and o == sorted(o)
    assert o[1] - o[0] >= 5 * R_pad * K_pad * 2                      # A digit planes
    wbp = -(-max(wb, lib.pg_chi0_prep_batch()) // wb) * wb          # frequencies per B-digit pass
    assert o[2] - o[1] >= wbp * 5 * R_pad * K_pad * 2                # B digit planes
    assert o[8] - o[7] >= nsplit * wb * npair * 128 * 128 * 8        # group-sum tiles
    assert lib.pg_chi0_mixed_workspace(nb1, nb2, nkp, npb, wb, kb_split) == o[8]


def test_chi0_prep_batch_setting():
    """Frequencies per B-digit pass: default 4, settable in [1, 64] (0 restores
    the default), whole GEMM batches, one set of five B planes per frequency
    in the workspace."""
    from pygw_gb300 import _lib
    lib = _lib.load()
    assert lib.pg_chi0_prep_batch() == 4
    args = (23, 192, 8, 300, 1, 0)
    base = lib.pg_chi0_mixed_workspace(*args)
    offs = (ctypes.c_size_t * 9)()
    dims = (ctypes.c_longlong * 9)()
    assert lib.pg_chi0_mixed_layout(*args, offs, dims) == 0
    plane = 5 * dims[3] * dims[1] * 2                                   # five planes of R_pad × K_pad bf16
    try:
        for bad in (-1, 65):
            assert lib.pg_set_chi0_prep_batch(bad) == -1
            assert lib.pg_chi0_prep_batch() == 4
        assert lib.pg_set_chi0_prep_batch(2) == 0 and lib.pg_chi0_prep_batch() == 2
        two = lib.pg_chi0_mixed_workspace(*args)
        assert base - two >= 2 * plane and base - two < 2 * plane + 4096 + 2 * 4 * dims[1] * 8
        # omega_batch 3 with a pass of 4: two whole launches, six frequencies
        assert lib.pg_set_chi0_prep_batch(4) == 0
        assert lib.pg_chi0_mixed_layout(23, 192, 8, 300, 3, 0, offs, dims) == 0
        assert offs[2] - offs[1] >= 6 * plane
    finally:
        lib.pg_set_chi0_prep_batch(0)
    assert lib.pg_chi0_prep_batch() == 4 and lib.pg_chi0_mixed_workspace(*args) == base


def test_weights_workspace_holds_scratch_and_records():
    """The weights workspace (host arithmetic): the scratch weights grow by
    4·ntet·P doubles per frequency of the chunk, and next to them sit the k
    lists, the per-chunk item arrays and the sub-tetrahedron records of one
    tetrahedron chunk (at most 1 GiB, at least one tetrahedron's worth: six
    records per band pair)."""
    from pygw_gb300 import _lib
    lib = _lib.load()
    nbnd, nkp, ncg, nomx, numin, nom, ntet = 200, 216, 0, 22, 8, 48, 1296     # C3: 23 × 192 band pairs
    P = (ncg + nomx + 1) * (nbnd - ncg - numin)
    per_omega = 4 * ntet * P * 8
    ws = [lib.pg_bz_calcqdepw_par2_workspace(nbnd, nkp, ncg, nomx, numin, nom, ntet, c) for c in (1, 2, 48)]
    assert ws[1] - ws[0] == per_omega and ws[2] - ws[0] == 47 * per_omega
    rest = ws[0] - per_omega
    assert 6 * P * 800 < rest <= (1 << 30) + (64 << 20)
    assert lib.pg_bz_calcqdepw_par2_workspace(nbnd, nkp, ncg, nomx, numin, nom, ntet, 0) == ws[2]
    # a small problem: the records of all its tetrahedra fit in one chunk
    small = lib.pg_bz_calcqdepw_par2_workspace(10, 8, 0, 3, 2, 4, 48, 0)
    assert 4 * 48 * 32 * 4 * 8 < small < 4 * 48 * 32 * 4 * 8 + 48 * 32 * 6 * 1024 + (1 << 16)


def test_polarization_entry_points_validate_on_the_host():
    """The weights, χ0 and ε⁻¹ entry points reject null pointers, inconsistent
    sizes and short workspaces before any device call (host code: runs without
    a GPU); their workspace queries return 0 for empty problems."""
    from pygw_gb300 import _lib
    lib = _lib.load()
    EARG, EWORK = -1, -2
    fake = 0x1000                     # never dereferenced: every call below fails its checks first
    big = 1 << 40
    # weights: nbnd 10, nkp 8, ncg 0, nomx 3, numin 2 (nb1 4, nb2 8), nom 4, ntet 48
    assert lib.pg_bz_calcqdepw_par2_workspace(10, 8, 0, 3, 10, 4, 48, 0) == 0          # nb2 = 0
    ww = lib.pg_bz_calcqdepw_par2_workspace(10, 8, 0, 3, 2, 4, 48, 0)
    assert ww > 0
    w8 = (None, 10, 8, 0.0, fake, 0, 3, 2, fake, 4, fake, 48, fake, fake, big, 0, None, None, None)
    assert lib.pg_bz_calcqdepw_par2(*w8) == EARG                                          # enk null
    assert lib.pg_bz_calcqdepw_par2(fake, *w8[1:11], 47, *w8[12:]) == EARG                # ntet != 6·nkp
    assert lib.pg_bz_calcqdepw_par2(fake, *w8[1:7], 10, *w8[8:]) == EARG                  # empty window
    assert lib.pg_bz_calcqdepw_par2(fake, *w8[1:14], ww - 1, *w8[15:]) == EWORK
    # FP64 χ0: k0 + nk beyond nkp, wings without their output
    c8 = (fake, 4, 0, fake, 3, 5, 5, 2, 16, -2.0, fake, None, None, None)
    assert lib.pg_chi0_accumulate_f64(None, *c8[1:]) == EARG
    assert lib.pg_chi0_accumulate_f64(fake, 4, 2, *c8[3:]) == EARG
    assert lib.pg_chi0_accumulate_f64(*c8[:11], fake, None, None) == EARG
    # split-precision χ0 (kb_split > 0: the layout needs no device query)
    assert lib.pg_chi0_mixed_workspace(3, 5, 0, 16, 2, 100) == 0
    wm = lib.pg_chi0_mixed_workspace(3, 5, 5, 16, 2, 100)
    m8 = (fake, 5, fake, 3, 5, 4, 16, -2.0, fake, fake, big, 2, 100, None, None, None)
    assert lib.pg_chi0_mixed(None, *m8[1:]) == EARG
    assert lib.pg_chi0_mixed(*m8[:11], 0, *m8[12:]) == EARG                               # omega_batch 0
    assert lib.pg_chi0_mixed(*m8[:10], wm - 1, *m8[11:]) == EWORK
    a8 = (fake, 2, 0, None, None, 0, fake, 3, 5, 5, 4, 16, -2.0, fake, 0, fake, big, 2, 100, None, None, None)
    assert lib.pg_chi0_mixed_accumulate(*a8[:2], 4, *a8[3:]) == EARG                      # k0 + nk > nkp
    assert lib.pg_chi0_mixed_accumulate(*a8[:3], fake, None, 20, *a8[6:]) == EARG          # kstart without knb2
    assert lib.pg_chi0_mixed_accumulate(*a8[:3], fake, fake, 31, *a8[6:]) == EARG          # nK > nk·nb1·nb2
    # ε⁻¹: q = 0 borders come together; refinement steps 0…2; workspace sizes
    assert lib.pg_eps_inverse_f64_workspace(0, 4) == 0 and lib.pg_eps_inverse_mixed_workspace(16, 0, 0) == 0
    wf = lib.pg_eps_inverse_f64_workspace(16, 4)
    assert lib.pg_eps_inverse_f64(fake, 16, 4, fake, None, fake, fake, big, None) == EARG
    assert lib.pg_eps_inverse_f64(fake, 16, 4, None, None, None, fake, wf - 1, None) == EWORK
    wx = lib.pg_eps_inverse_mixed_workspace(16, 4, 0)
    assert lib.pg_eps_inverse_mixed(fake, 16, 4, None, None, None, fake, big, 0, 3, None, None) == EARG
    assert lib.pg_eps_inverse_mixed(fake, 16, 4, None, None, None, fake, wx - 1, 0, 2, None, None) == EWORK
    assert lib.pg_eps_inverse_mixed_workspace(16, 4, 2) < wx                               # two frequencies at a time


def test_batch_tuner_keeps_the_fastest_choice_per_shape_class(tmp_path):
    """The batch autotuner (host logic): the fastest candidate per shape class
    wins, is written to the JSON file, and a tuner loaded from that file
    returns it without timing anything again; the key bins N to 256 and K to
    65,536 so nearby shapes share a choice."""
    from pygw_gb300.batch import Tuner
    path = str(tmp_path / "tune.json")
    times = {(8, 1): 5.0, (8, 2): 3.0, (16, 2): 4.0}
    seen = []

    def timer(kc, wb):
        seen.append((kc, wb))
        return times[(kc, wb)]

    t = Tuner(path)
    key = Tuner.key(1200, 23, 192, 216, 953856, 48)
    assert key == Tuner.key(1100, 23, 192, 216, 953856 - 1000, 48) != Tuner.key(1300, 23, 192, 216, 953856, 48)
    c = t.choose(key, list(times), timer)
    assert (c.k_chunk, c.omega_batch, c.ms_per_omega) == (8, 2, 3.0) and seen == list(times)

    def no_timer(kc, wb):
        raise AssertionError("a stored choice must not be timed again")

    c2 = Tuner(path).choose(key, list(times), no_timer)
    assert (c2.k_chunk, c2.omega_batch) == (8, 2)


def test_mixed_omega_batch_is_the_fewest_frequencies_filling_two_waves():
    """Host logic of the split-precision frequency batch: the fewest
    frequencies per launch (doubling) whose work units fill two waves of
    2-CTA clusters on 152 SMs, within the memory budget.  At C3 (55 blocks ×
    4 K splits) one frequency already gives 220 units; a small problem needs
    more frequencies; a tight budget stops the doubling."""
    from pygw_gb300 import eps as peps
    big = 1 << 45
    assert peps.mixed_omega_batch(23, 192, 216, 1200, 48, budget_bytes=big, sm_count=152) == 1
    wb_small = peps.mixed_omega_batch(9, 24, 8, 128, 16, budget_bytes=big, sm_count=152)
    assert wb_small > 1 and wb_small & (wb_small - 1) == 0 and wb_small <= 16
    from pygw_gb300 import _lib
    lib = _lib.load()
    tight = lib.pg_chi0_mixed_workspace(9, 24, 8, 128, 2, 0)           # room for one doubling only
    assert peps.mixed_omega_batch(9, 24, 8, 128, 16, budget_bytes=tight, sm_count=152) == min(2, wb_small)
    assert peps.mixed_omega_batch(9, 24, 8, 128, 3, budget_bytes=big, sm_count=152) <= 3
