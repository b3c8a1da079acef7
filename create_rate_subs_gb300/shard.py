"""Splitting a batch of states across ranks.

States are independent, so N GPUs each evaluate one contiguous slab of the
structure-of-arrays batch with a replica of the mechanism tables; no
collective is needed on the data path (bench.py runs one slab per rank and
reports weak scaling).
"""

__all__ = ["shard_range"]


def shard_range(n_states, rank, world):
    """[begin, end) of the states rank ``rank`` of ``world`` evaluates:
    contiguous slabs whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world %r/%r" % (rank, world))
    if n_states < 0:
        raise ValueError("n_states < 0")
    base, extra = divmod(n_states, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)
