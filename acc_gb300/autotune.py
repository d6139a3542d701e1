"""Launch-shape autotuner for the fused kernels.

For a workload it times a short sample under each candidate launch shape
(threads per block, resident blocks per SM, work-item size for the batched
launch) with CUDA events, keeps the fastest, and caches the choice in a
JSON file keyed by GPU name, chain signature (the opcodes) and precision.
Tallies touched by the trial runs are restored afterwards, so tuning does
not change results.
"""

import json
import os
import threading

from . import engine

CACHE = os.environ.get(
    "ACC_GB300_AUTOTUNE_CACHE",
    os.path.join(os.path.expanduser("~"), ".cache", "acc_gb300",
                 "autotune.json"))

_lock = threading.Lock()


def _signature(instruments, floattype, kind):
    import torch
    ops = []
    for ins in instruments[:1]:
        ops = [int(c.opcode) for c in ins.components]
    return "|".join([torch.cuda.get_device_name(), kind, str(floattype),
                     ",".join(map(str, ops)), str(len(instruments))])


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    with _lock:
        d = _load()
        d[key] = value
        try:
            os.makedirs(os.path.dirname(CACHE), exist_ok=True)
            tmp = CACHE + ".tmp"
            with open(tmp, "w") as f:
                json.dump(d, f, indent=1)
            os.replace(tmp, CACHE)
        except OSError:
            pass


def _tallies(instruments):
    out = []
    for ins in instruments:
        for c in ins.components:
            t = getattr(c, "_device_tally", None)
            if t is not None:
                out.append(t)
    return out


def _time(fn, reps=2):
    import torch
    fn()  # warm-up
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    engine.read_status()
    return best


def tune_batched(instruments, counts, seeds, floattype="float32",
                 fraction=0.05, candidates=None, use_cache=True):
    """Best (threads_per_block, blocks, chunk) for a batched run, timed on
    `fraction` of each variant's neutrons."""
    import torch
    key = _signature(instruments, floattype, "batched")
    if use_cache:
        hit = _load().get(key)
        if hit:
            return hit
    sms = torch.cuda.get_device_properties(
        torch.cuda.current_device()).multi_processor_count
    if candidates is None:
        candidates = [(t, k, ch) for t in (128, 256) for k in (2, 4, 8)
                      for ch in (2048, 8192, 32768)]
    small = [max(1, int(c * fraction)) for c in counts]
    for ins in instruments:  # bind tallies before saving them
        engine.chain_for_instrument(ins)
    saved = [t.clone() for t in _tallies(instruments)]
    results = []
    for tpb, per_sm, chunk in candidates:
        blocks = sms * per_sm * (256 // tpb)
        ms = _time(lambda: engine.run_batched(
            instruments, small, seeds, floattype=floattype,
            threads_per_block=tpb, blocks=blocks, chunk=chunk, sync=False))
        results.append((ms, tpb, blocks, chunk))
    for t, s in zip(_tallies(instruments), saved):
        t.copy_(s)
    ms, tpb, blocks, chunk = min(results)
    best = {"threads_per_block": tpb, "blocks": blocks, "chunk": chunk,
            "trial_ms": ms, "trials": len(results)}
    _store(key, best)
    return best


def tune_chain(instrument, ncount, floattype="float32", candidates=None,
               use_cache=True):
    """Best (threads_per_block, blocks) for the single-instrument kernel."""
    import torch
    key = _signature([instrument], floattype, "chain")
    if use_cache:
        hit = _load().get(key)
        if hit:
            return hit
    sms = torch.cuda.get_device_properties(
        torch.cuda.current_device()).multi_processor_count
    if candidates is None:
        candidates = [(t, k) for t in (128, 256) for k in (2, 4, 6, 8, 16)]
    chain = engine.chain_for_instrument(instrument)
    saved = [t.clone() for t in _tallies([instrument])]
    results = []
    for tpb, per_sm in candidates:
        blocks = sms * per_sm * (256 // tpb)
        ms = _time(lambda: engine.run_chain(
            chain, ncount, floattype=floattype, threads_per_block=tpb,
            blocks=blocks, sync=False))
        results.append((ms, tpb, blocks))
    for t, s in zip(_tallies([instrument]), saved):
        t.copy_(s)
    ms, tpb, blocks = min(results)
    best = {"threads_per_block": tpb, "blocks": blocks, "trial_ms": ms,
            "trials": len(results)}
    _store(key, best)
    return best
