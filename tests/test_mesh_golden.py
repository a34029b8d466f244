"""The product's tetrahedra and k − q table against golden vectors from the
reference's own KQmesh.tetra (kqmesh.py:188-380), run by
tests/golden/make_mesh_golden.py on several meshes and reciprocal bases that
make each of the four cube diagonals the shortest.  The corner order of every
tetrahedron matters: the weights are assigned per corner."""
import os

import numpy as np
import pytest

from pygw_gb300.mesh import build_kqid, build_tetc, shortest_diagonal

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mesh_golden.npz"))
CASES = sorted({k.split(".")[0] for k in GOLDEN.files})


@pytest.mark.parametrize("case", CASES)
def test_tetrahedra_and_kqid_match_the_reference_code(case):
    g = lambda k: GOLDEN[f"{case}.{k}"]  # noqa: E731
    div, gbas = g("div"), g("gbas")
    assert shortest_diagonal(div, gbas) == int(g("mnd"))
    assert np.array_equal(build_tetc(div, gbas), g("tetc"))
    assert np.array_equal(build_kqid(div), g("kqid"))


def test_the_cases_cover_every_diagonal():
    assert {int(GOLDEN[f"{c}.mnd"]) for c in CASES} == {0, 1, 2, 3}


def test_weight_energies_match_the_reference_code():
    """The energies Polarization_weights hands the weight kernel (core states
    first, then the bands of each k-point's irreducible point), against the
    arguments the reference's own Polarization_weights passes to its Fortran
    routines (tests/golden/make_polarization_weights_golden.py)."""
    from pygw_gb300.polarization import assemble_enk
    G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "polarization_weights_golden.npz"))

    class NS:
        def __init__(self, **kw):
            self.__dict__.update(kw)
    ks = NS(ncg_p=int(G["ncg_p"]), nbmaxpol=int(G["nbmaxpol"]), Ebnd=G["Ebnd"])
    kqm = NS(kii_ind=G["kii_ind"])
    core = NS(corind=G["corind"], eig_core=[[list(G["eig_core0"]), list(G["eig_core1"])]])
    enk = assemble_enk(ks, kqm, core)
    assert np.array_equal(enk, G["enk"]) and np.array_equal(enk, G["enk_par3"])
    assert np.array_equal(G["kqid_par2"], G["kqid"][:, 1]) and np.array_equal(G["kqid_par3"], G["kqid"][:, 0])
