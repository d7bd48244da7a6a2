"""Row partitioning of the stage across ranks.

The kNN, the weights and the per-row CSR gather are independent per query row,
so N rows split into contiguous blocks, one per rank, with no exchange until the
neighbour table is complete; M's rows then need the gathered (idx, W) table
(one all-gather). Used by bench.py for multi-GPU runs (each rank times its own
block) and by the gloo tests.
"""


def shard_rows(n: int, rank: int, world: int):
    """[lo, hi) of the rows owned by `rank` (blocks differ by at most one row)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi
