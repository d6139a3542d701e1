"""Several GPUs: split the neutron index range, sum the tallies once.

Neutron i draws from the Philox stream (seed, i) whatever device runs it,
so ranks that take disjoint index ranges and add their (N, sum p, sum p^2)
tallies reproduce the single-device run up to the order of floating-point
additions.  There is no exchange during propagation; the only collectives
are one all-reduce of the tallies at the end and, for a differentiable run,
one of the gradients (torch.distributed: NCCL between GPUs, gloo on CPUs).
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


def reduce_gradients(grads, group=None):
    """Sum a {name: tensor} gradient dictionary over all ranks in place:
    the gradient of a sum over neutrons is the sum of the ranks' gradients
    over their neutron blocks.  Returns the dictionary."""
    import torch
    import torch.distributed as dist
    for name in sorted(grads):
        t = grads[name]
        if not isinstance(t, torch.Tensor):
            t = grads[name] = torch.as_tensor(t, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return grads


def engine_runner(seed=None, floattype=None):
    """The runner run_sharded uses by default: the fused kernel on the
    current GPU over the neutron block [first, first + count); returns
    (processed, the monitors' device tallies)."""
    def run(instrument, first, count):
        from . import engine
        from .components.monitors.MonitorBase import MonitorBase
        chain = engine.chain_for_instrument(instrument)
        st = engine.run_chain(chain, count, seed=seed, floattype=floattype,
                              first=first)
        tallies = [c._device_tally for c in instrument.components
                   if isinstance(c, MonitorBase)
                   and getattr(c, "_device_tally", None) is not None]
        return int(st.processed), tallies
    return run


def run_sharded(instrument, ncount, rank, world, seed=None, floattype=None,
                group=None, runner=None):
    """Run this rank's share of `ncount` neutrons and all-reduce every
    monitor's tally; returns the processed count of this rank.  `runner`
    (instrument, first, count) -> (processed, tally tensors) does the
    propagation: engine_runner(seed, floattype) by default, the fused
    kernel on the current GPU."""
    first, count = shard_range(ncount, rank, world)
    if runner is None:
        runner = engine_runner(seed, floattype)
    processed, tallies = runner(instrument, first, count)
    reduce_tallies(tallies, group)
    return int(processed)


def merge_host_tallies(parts):
    """Sum per-rank host tallies (list of dicts id -> array)."""
    out = {}
    for p in parts:
        for k, v in p.items():
            out[k] = out.get(k, 0) + np.asarray(v)
    return out
