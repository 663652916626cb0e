"""Splitting one event across ranks (GPUs) and putting its hits back together.

Photons are independent and each one's random stream is fixed by its event-level index (the subsequence of
qudarap/qrng.h:131-137 is the photon index, offset by photon_slot_offset for sliced launches, CSGOptiX7.cu:415),
so an event can be cut at any genstep boundary: rank r simulates a contiguous range of gensteps with the event
photon offset of its first photon, and the event's hits are the ranks' hits concatenated in rank order.  There is
no exchange during simulation; only the final hit gather.
"""
import numpy as np


def photon_counts(gs):
    return np.ascontiguousarray(gs).view(np.uint32).reshape(-1, 24)[:, 3].astype(np.int64)


def shard_ranges(gs, world):
    """Contiguous genstep ranges [g0, g1) per rank with about equal photon counts, and each range's photon offset."""
    counts = photon_counts(gs)
    ends = np.cumsum(counts)
    total = int(ends[-1]) if len(ends) else 0
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        bounds.append(int(np.searchsorted(ends, target, side="left")) + 1 if total else 0)
    bounds.append(len(gs))
    bounds = np.maximum.accumulate(np.clip(bounds, 0, len(gs)))
    out = []
    for r in range(world):
        g0, g1 = int(bounds[r]), int(bounds[r + 1])
        offset = int(ends[g0 - 1]) if g0 > 0 else 0
        out.append((g0, g1, offset))
    return out


def shard_gensteps(gs, rank, world):
    """This rank's gensteps and the event photon offset of its first photon."""
    g0, g1, offset = shard_ranges(gs, world)[rank]
    return gs[g0:g1], offset


def merge_hits(parts):
    """Event hits in photon order from the ranks' hits (rank order is photon order)."""
    parts = [p for p in parts if len(p)]
    return np.concatenate(parts) if parts else np.zeros(0, dtype=parts[0].dtype if parts else None)


def simulate_sharded(engine, event_id, gs, rank, world, dist=None):
    """Simulate this rank's share of an event with the engine; rank 0 returns the whole event's hits."""
    part, offset = shard_gensteps(gs, rank, world)
    engine.simulate_slice(event_id, part, offset)
    hits = engine.hits()
    if dist is None or world == 1:
        return hits
    gathered = [None] * world
    dist.all_gather_object(gathered, hits)
    return merge_hits(gathered) if rank == 0 else None
