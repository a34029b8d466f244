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
