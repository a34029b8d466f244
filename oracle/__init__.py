"""Oracle: CPU restatements of the reference's polarization path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, and only as the checker or the timed CPU baseline.

Parity unpinned: the reference ships no tests, fixtures or golden vectors for this
path and cannot be built or run here (Fortran without a compiler, Python 2 with
f2py modules); this restatement is pinned by known answers instead
(tests/test_oracle_*.py).
"""
