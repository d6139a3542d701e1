"""Several GPUs: split the neutron index range, sum the tallies once.

Neutron i draws from the Philox stream (seed, i) whatever device runs it,
so ranks that take disjoint index ranges and add their (N, sum p, sum p^2)
tallies reproduce the single-device run up to the order of floating-point
additions.  There is no exchange during propagation; the only collective is
one all-reduce of the tallies at the end (torch.distributed: NCCL between
GPUs, gloo on CPUs).
"""

import numpy as np


def shard_range(ncount, rank, world):
    """(first, count) of rank's contiguous block of [0, ncount)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(int(ncount), int(world))
    first = rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return first, count


def reduce_tallies(tensors, group=None):
    """Sum tally tensors over all ranks in place."""
    import torch.distributed as dist
    for t in tensors:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return tensors


def run_sharded(instrument, ncount, rank, world, seed=None, floattype=None,
                group=None):
    """Run this rank's share of `ncount` neutrons on the current GPU and
    all-reduce every monitor's tally; returns the processed count of this
    rank."""
    from . import engine
    from .components.monitors.MonitorBase import MonitorBase
    first, count = shard_range(ncount, rank, world)
    chain = engine.chain_for_instrument(instrument)
    st = engine.run_chain(chain, count, seed=seed, floattype=floattype,
                          first=first)
    tallies = [c._device_tally for c in instrument.components
               if isinstance(c, MonitorBase)
               and getattr(c, "_device_tally", None) is not None]
    reduce_tallies(tallies, group)
    return int(st.processed)


def merge_host_tallies(parts):
    """Sum per-rank host tallies (list of dicts id -> array)."""
    out = {}
    for p in parts:
        for k, v in p.items():
            out[k] = out.get(k, 0) + np.asarray(v)
    return out
