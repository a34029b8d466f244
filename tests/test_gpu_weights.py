"""GPU tetrahedron weights vs the oracle — bit-exact (sm_103a, through the C-ABI)."""
import numpy as np
import pytest
import torch

from oracle import weights as ow
from pygw_gb300 import polarization as pol
from pygw_gb300.synthetic import WORKLOADS, Problem, scaled

pytestmark = pytest.mark.gpu


def _args(p, iq=None):
    b = p.bands
    nomx, numin = b.nomax_numin
    iq = p.qs[0] if iq is None else iq
    return (b.enk(), b.EF, p.kqm.kqid[:, iq], 0, nomx, numin, p.fr.omega, p.kqm.tetc)


def _compare(args, nom_chunk=0):
    ref, st_ref, stats = ow.bz_calcqdepw_par2(*args, return_stats=True)
    r = pol.weights_device(*args, nom_chunk=nom_chunk)
    torch.cuda.synchronize()
    got = r.numpy()
    assert got.shape == ref.shape
    assert r.status == st_ref
    assert r.counters == stats
    diff = np.abs(got - ref)
    assert np.array_equal(got, ref), f"max |Δ| = {diff.max():.3e} (max |w| {np.abs(ref).max():.3e})"
    return got


def test_c1_bit_exact():
    _compare(_args(Problem(WORKLOADS["C1"])))


def test_c1_all_q_bit_exact():
    p = Problem(WORKLOADS["C1"])
    for iq in (0, 5, 21, 63):
        _compare(_args(p, iq))


def test_c2_one_q_bit_exact():
    _compare(_args(Problem(WORKLOADS["C2"])))


def test_c3_mesh_reduced_bands_bit_exact():
    w = scaled(WORKLOADS["C3"], nbands=48, nom=12)
    _compare(_args(Problem(w)))


def test_frequency_chunks_do_not_change_bits():
    p = Problem(WORKLOADS["C1"])
    a = _compare(_args(p), nom_chunk=0)
    b = pol.weights_device(*_args(p), nom_chunk=5).numpy()
    assert np.array_equal(a, b)


def test_degenerate_inputs_match_oracle():
    """Energies exactly at EF, flat (fully grouped) bands, equal corner values."""
    p = Problem(scaled(WORKLOADS["C1"], div=3, nbands=10, nocc=4, nom=8))
    args = list(_args(p))
    enk = args[0].copy()
    ef = args[1]
    enk[2, ::2] = ef                      # a band touching EF at half the points
    enk[5, :] = enk[5, 0]                 # a flat band
    enk[6, 3] = enk[6, 4] = enk[6, 5]     # equal corner energies
    args[0] = np.asfortranarray(enk)
    _compare(tuple(args))


def test_random_partial_occupation_stress():
    rng = np.random.default_rng(11)
    p = Problem(scaled(WORKLOADS["C1"], div=3, nbands=12, nocc=5, nom=6))
    args = list(_args(p))
    enk = np.asfortranarray(args[1] + rng.uniform(-1.5, 1.5, args[0].shape) + np.linspace(-1, 1, 12)[:, None])
    args[0] = enk
    _compare(tuple(args))


def test_drop_in_polarization_weights():
    p = Problem(WORKLOADS["C1"])
    iq = p.qs[0]
    got = pol.Polarization_weights(iq, p.bands, p.kqm, None, p.fr, 0, 3, None, None)
    ref = ow.bz_calcqdepw_par2(*_args(p, iq))
    assert got.flags.f_contiguous and np.array_equal(got, ref)


def test_repeatable():
    p = Problem(WORKLOADS["C1"])
    a = pol.weights_device(*_args(p)).numpy()
    b = pol.weights_device(*_args(p)).numpy()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["c1", "stress"])
def test_against_the_reference_statements(name):
    """The GPU weights against kcw from the reference's own Fortran statements
    (tests/golden/weights_golden.npz, portable atan/log): bit-identical
    everywhere except the kcw entries of 7- and 8-node items from the third
    frequency on, where the reference's wtemp(4,2,nom) layout aliases the two
    halves of the polyhedron (see tests/test_oracle_weights_golden.py)."""
    from test_oracle_weights_golden import alias_mask, item_nodes, load_case
    a, ref = load_case(name)
    r = pol.weights_device(a["enk"], a["ef"], a["kqid"], a["ncg"], a["nomx"], a["numin"], a["omega"], a["tetc"])
    torch.cuda.synchronize()
    assert r.status == 0
    got = r.numpy()
    want = ref["portable"]
    assert got.shape == want.shape
    diff = got != want
    mask = alias_mask(a, item_nodes(a))
    assert not np.any(diff & ~mask), np.argwhere(diff & ~mask)[:5]


@pytest.mark.parametrize("name", ["c1", "stress"])
def test_reference_layout_matches_every_entry(name):
    """With the reference's wtemp addressing reproduced
    (pg_set_weights_reference_layout), the GPU weights equal the reference's
    statements at every kcw entry, the frequency-chunked evaluation included."""
    from test_oracle_weights_golden import load_case
    a, ref = load_case(name)
    with pol.reference_layout():
        for chunk in (0, 1):
            r = pol.weights_device(a["enk"], a["ef"], a["kqid"], a["ncg"], a["nomx"], a["numin"], a["omega"],
                                   a["tetc"], nom_chunk=chunk)
            torch.cuda.synchronize()
            assert r.status == 0
            got = r.numpy()
            assert np.array_equal(got, ref["portable"]), (chunk, np.abs(got - ref["portable"]).max())
    # and back to the default afterwards
    r = pol.weights_device(a["enk"], a["ef"], a["kqid"], a["ncg"], a["nomx"], a["numin"], a["omega"], a["tetc"])
    torch.cuda.synchronize()
    assert np.array_equal(r.numpy(), ow.bz_calcqdepw_par2(a["enk"], a["ef"], a["kqid"], a["ncg"], a["nomx"],
                                                         a["numin"], a["omega"], a["tetc"]))
