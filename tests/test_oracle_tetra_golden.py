"""The oracle's per-tetrahedron weights against the reference's own statements (CPU).

``tests/golden/tetra_golden.npz`` holds, for 1100 seeded corner-energy sets (e
occupied, f empty, EF = 0; energies on a grid of 0.25, pairs 0 to 0.25 apart,
continuous values, and f - e equal or nearly equal across the corners), what
the reference's ``convw1t_par`` and its callees (for_tetrahedra3.f90:3-743,
for_tetrahedra2.f90:1688-2773) compute when executed from their Fortran text by
``tests/golden/make_tetra_golden.py``, at six imaginary frequencies including 0
and 1e-7: the 4 × nom corner weights, or the verdict that their result is
undefined in compiled code (storage never written, a subscript beyond an array,
a bit test at an unset position) or that they call ``stop``, and where. The
corner sets cover every polyhedron node count and every branch of ``sortnodes``
that orders well-defined polyhedra.
"""
import os

import numpy as np
import pytest

from oracle import weights as ow

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "tetra_golden.npz")
ERR_UNDEFINED = 1 << 5


@pytest.fixture(scope="module")
def golden():
    g = np.load(GOLDEN)
    return {k: g[k] for k in g.files}


def _run(g, i):
    return ow.convw1t(g["e"][i], g["f"][i], 0.0, g["omega"])


def test_well_defined_tetrahedra_match_bit_for_bit(golden):
    """With the reference's wtemp addressing for 7- and 8-node polyhedra,
    every weight of every well-defined tetrahedron is bit-identical."""
    g = golden
    ok = np.flatnonzero(g["kind"] == 0)
    assert len(ok) > 800
    nnods = []
    with ow.reference_layout():
        for i in ok:
            w, st, nn = _run(g, i)
            assert st == 0, (i, st)
            assert np.array_equal(w, g["weight"][i]), (i, g["e"][i], g["f"][i], np.abs(w - g["weight"][i]).max())
            nnods.append(nn)
    counts = np.bincount(nnods, minlength=9)
    assert all(counts[n] > 0 for n in range(3, 9)), counts


def test_well_defined_tetrahedra_match_with_the_c_library_atan_log(golden):
    """The same statements with the C library's atan/log (what a compiled
    reference calls) against the oracle built with them: bit for bit too."""
    g = golden
    with ow.reference_layout():
        for i in np.flatnonzero(g["kind"] == 0):
            w, st, _ = ow.convw1t(g["e"][i], g["f"][i], 0.0, g["omega"], libm=True)
            assert st == 0 and np.array_equal(w, g["weight_libm"][i]), i


def test_default_layout_differs_only_where_the_halves_alias(golden):
    """Without the reference's layout the oracle adds the two halves of a
    7- or 8-node polyhedron at every frequency; it then differs from the
    statements only at those polyhedra, from the third frequency on."""
    g = golden
    aliased = 0
    for i in np.flatnonzero(g["kind"] == 0):
        w, st, nn = _run(g, i)
        d = w != g["weight"][i]
        if nn < 7:
            assert not d.any(), i
        else:
            assert not d[:, :2].any(), i
            aliased += bool(d.any())
    assert aliased > 0


# the oracle's bit for each of the reference's stop sites (make_tetra_golden.STOP_SITES):
# sortnodes' two messages, convw1t_par's 'error in setnodes' after relnodes or
# sortnodes report a failure, sorteq, convw1t_par's node count, stweight_imag_par
SITE_BITS = {1: 1 << 2, 2: 1 << 2, 3: (1 << 2) | (1 << 3), 4: 1 << 1, 5: 1 << 0, 6: 1 << 4}


def test_undefined_and_stopping_tetrahedra_are_flagged(golden):
    """Where the statements' result is undefined (storage never written, a
    subscript beyond an array, a bit test at an unset position) the oracle
    reports PG_ERR_UNDEFINED; where they call stop from defined values it
    reports that stop site's condition and nothing undefined."""
    g = golden
    k = g["kind"]
    assert (k == 1).sum() >= 20 and (k == 2).sum() >= 5
    for i in np.flatnonzero(k == 1):
        _, st, _ = _run(g, i)
        assert st & ERR_UNDEFINED, (i, st)
    for i in np.flatnonzero(k == 2):
        _, st, _ = _run(g, i)
        assert st & SITE_BITS[int(g["stop_site"][i])] and not st & ERR_UNDEFINED, (i, st, g["stop_site"][i])


def test_static_limit_branches_are_present(golden):
    """The fixture reaches ω = 0 (the arc tangent's limit ±π/2), weights
    beyond the unphysical tolerance zeroed below |ω| = 1e-6, and finite
    weights there."""
    g = golden
    ok = g["kind"] == 0
    w = g["weight"][ok]
    assert g["omega"][0] == 0.0 and np.isfinite(w).all()
    assert np.count_nonzero(w[:, :, 0]) > 100


def test_well_defined_tetrahedra_through_the_mesh_driver(golden):
    """The same corner sets embedded in a mesh and run through the oracle's
    bz_calcqdepw_par2 (for_tetrahedra.f90:390-464): one tetrahedron per four
    k-points with the occupied band as band 0 and the empty one as band 1,
    k − q = k, and filler tetrahedra (ntet = 6·nkp, as the driver's tetln
    requires) on four extra k-points where both bands lie below EF, so that
    every filler item is skipped.  Each k-point then holds one corner's
    weight times 6·wtet, formed as the driver forms it: (w·6)·(1/ntet)."""
    g = golden
    ok = np.flatnonzero(g["kind"] == 0)
    n = len(ok)
    nkp = 4 * n + 4
    ntet = 6 * nkp
    enk = np.full((2, nkp), -1.0)
    enk[0, :4 * n] = g["e"][ok].ravel()
    enk[1, :4 * n] = g["f"][ok].ravel()
    tetc = np.full((4, ntet), 4 * n, dtype=np.int32) + np.arange(4, dtype=np.int32)[:, None]
    tetc[:, :n] = 4 * np.arange(n)[None, :] + np.arange(4)[:, None]
    om = g["omega"]
    with ow.reference_layout():
        kcw, st, _ = ow.bz_calcqdepw_par2(np.asfortranarray(enk), 0.0, np.arange(nkp), 0, 0, 1, om,
                                          np.asfortranarray(tetc), return_stats=True)
    want = np.zeros((nkp, len(om)))
    want[:4 * n] = ((g["weight"][ok] * 6.0) * (1.0 / ntet)).reshape(4 * n, len(om))
    assert st == 0 and kcw.shape == (1, 1, nkp, len(om))
    assert np.array_equal(kcw[0, 0], want)


def test_one_frequency_seven_and_eight_node_halves_are_undefined_in_the_reference_layout(golden):
    """convw1t_par's wtemp(4,2,nom) holds 8·nom values and the second half of
    a 7- or 8-node polyhedron is written from the 9th on (for_tetrahedra3.f90:
    36, 100-120): with one frequency that lies past the array's end, which is
    undefined in compiled code; the oracle then flags it (reference layout
    only) and adds the halves.  With two frequencies it is defined."""
    g = golden
    big = [i for i in np.flatnonzero(g["kind"] == 0) if _run(g, i)[2] >= 7][:20]
    assert big
    for i in big:
        for nom, flagged in ((1, True), (2, False)):
            om = g["omega"][3:3 + nom]
            with ow.reference_layout():
                w, st, _ = ow.convw1t(g["e"][i], g["f"][i], 0.0, om)
            w0, st0, _ = ow.convw1t(g["e"][i], g["f"][i], 0.0, om)
            assert bool(st & ERR_UNDEFINED) == flagged and st0 == 0
            assert np.array_equal(w, w0)
