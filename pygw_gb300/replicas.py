"""q points over ranks: one process per GPU, no collective on the data path.

The reference splits the q list over MPI ranks with ``mpiSplitArray``
(mcommon.py:423-454; used at pygw.py:3654-3659): contiguous blocks of
ceil(nq/size) points, and when there are more ranks than points, ranks in
steps of (size+1)//nq take one point each while the others take none.  Each
rank then runs its q points independently; the only reduction is the sum of
the self-energy arrays at the end (pygw.py:3717-3718).
"""
from __future__ import annotations

import numpy as np


def split_range(rank: int, size: int, n: int):
    """(start, end) of the block of ``n`` items that ``rank`` of ``size`` takes."""
    if n <= 0:
        return 0, 0
    per = n // size if n % size == 0 else n // size + 1
    if size <= n:
        return min(rank * per, n), min((rank + 1) * per, n)
    step = (size + 1) // n
    if rank % step == 0 and rank // step < n:
        return rank // step, rank // step + 1
    if rank // step < n:
        return rank // step, rank // step
    return n - 1, n - 1


def split(rank: int, size: int, n: int):
    """(start, end, counts[size], displacements[size]) as the reference returns them."""
    counts, displ = [], []
    for r in range(size):
        s, e = split_range(r, size, n)
        counts.append(e - s)
        displ.append(s)
    s, e = split_range(rank, size, n)
    return s, e, np.array(counts, dtype=int), np.array(displ, dtype=int)


def my_points(points, rank: int, size: int):
    """The items of ``points`` this rank runs."""
    s, e = split_range(rank, size, len(points))
    return list(points[s:e])
