"""Frame-range sharding of one long request across ranks (one GPU each).

Frames are independent: rank r computes frames [f0, f1) from the signal
slice [f0*hop, min(n, (f1-1)*hop + N)) (a halo of N - hop samples) and owns
output rows [f0, f1).  No exchange step and no collective is needed; the
caller concatenates the rows.  Row layouts shard this way: power in the
reference layout (N floats per frame) and both dense layouts (N/2+1 bins per
frame).  The reference's flat half-complex layout spans frame boundaries and
is produced whole on one device.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass(frozen=True)
class Shard:
    rank: int
    f0: int          # first frame (inclusive)
    f1: int          # last frame (exclusive)
    s0: int          # first input sample of the slice
    s1: int          # end of the input slice (exclusive)
    row: int         # output floats per frame


def row_floats(n_window: int, options: str) -> int:
    if "--layout=dense" in options:
        return (n_window // 2 + 1) * (2 if "--half_complex_return" in options else 1)
    if "--half_complex_return" in options:
        raise ValueError("the flat half-complex layout does not shard by frame rows")
    return n_window


def plan(n: int, qt: int, hop: int, n_window: int, options: str, world: int) -> list[Shard]:
    """Split qt frames into `world` contiguous ranges of near-equal size."""
    row = row_floats(n_window, options)
    out = []
    for r in range(world):
        f0 = qt * r // world
        f1 = qt * (r + 1) // world
        s0 = min(n, f0 * hop)
        s1 = min(n, max(s0, (f1 - 1) * hop + n_window)) if f1 > f0 else s0
        out.append(Shard(r, f0, f1, s0, s1, row))
    return out


def slice_rows(result_of_slice, shard: Shard):
    """Rows [f0, f1) out of the output of the slice request (its frame j is frame f0 + j)."""
    return result_of_slice[: (shard.f1 - shard.f0) * shard.row]
