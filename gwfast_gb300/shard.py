"""Replicas over event shards for several GPUs (one process per GPU).

Events are independent, so a catalogue is split into contiguous shards, each rank
evaluates its shard on its own GPU, and the results are concatenated.  There is no
data-path collective; the gather at the end is a host-side object gather.
"""
import numpy as np


def shard_slice(n, rank, world):
    """Contiguous [start, stop) of rank `rank` among `world` for n events (sizes differ by at most 1)."""
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_events(events, rank, world):
    n = len(np.atleast_1d(events['Mc']))
    a, b = shard_slice(n, rank, world)
    return {k: (np.atleast_1d(v)[a:b] if np.ndim(v) else v) for k, v in events.items()}


def run_sharded(fn, events, rank, world, group=None):
    """Evaluate fn(events_shard) -> array with events on the last axis on every rank; return the full result."""
    import torch.distributed as dist
    part = fn(shard_events(events, rank, world))
    if world == 1:
        return part
    parts = [None] * world
    dist.all_gather_object(parts, part, group=group)
    return np.concatenate(parts, axis=-1)
