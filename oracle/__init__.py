"""Oracle: CPU restatements of the reference's polarization path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, and only as the checker or the timed CPU baseline.

Parity: the reference ships no tests or golden vectors and its driver (Python 2
with f2py modules) cannot be imported.  Its numpy parts — calc_eps and the
Python around the self-energy convolutions — are run from their source text on
seeded inputs by the scripts in tests/golden/, and the restatements here
reproduce those outputs (tests/test_*golden.py).  Its Fortran parts —
the tetrahedron weights and the convolution kernels — cannot be built (no
Fortran compiler); their restatements are pinned by known answers
(tests/test_oracle_*.py).
"""
