"""Host side of the engine: assemble an mcv_chain from components and call
the C ABI (include/acc_gb300.h) through ctypes.

Device memory (tallies, tables, neutron arrays) is allocated with torch;
only raw pointers cross into the library.
"""

import ctypes

import numpy as np

from . import _native as nat
from . import config
from .instrument import calcTransformations


def build_chain(components, offsets=None, rotmats=None, binder=None):
    """An mcv_chain for `components`, with the frame transforms between
    consecutive components (identity when offsets/rotmats are None).  A
    component with extra slots (a sample with a composite kernel) is
    followed by them; they take the identity transform, and the next
    component the transform from the component they follow."""
    extra = [int(getattr(c, "extra_slots", lambda: 0)()) for c in components]
    nslots = len(components) + sum(extra)
    if not components or not 1 <= nslots <= nat.MCV_MAX_COMPONENTS:
        raise ValueError(
            f"a chain holds 1..{nat.MCV_MAX_COMPONENTS} components "
            f"(composite kernel elements included), got {nslots}")
    if binder is None:
        from .memory import DeviceBinder
        binder = DeviceBinder()
    ch = nat.mcv_chain()
    # the chain holds raw pointers into memory that the binder and the
    # components own (tallies, lookup tables): keep both alive with it, so
    # that a chain built from a temporary instrument stays valid
    ch._binder = binder
    ch._components = list(components)
    ch.ncomp = nslots
    eye = np.eye(3)

    def transform(slot, off, rot):
        for k in range(9):
            ch.rot[slot][k] = float(rot.flat[k])
            ch.frot[slot][k] = float(rot.flat[k])
        for k in range(3):
            ch.off[slot][k] = float(off[k])
            ch.foff[slot][k] = float(off[k])
        if np.array_equal(rot, eye):
            ch.comp[slot].flags |= nat.FLAG_IDENTITY_ROT

    slot = 0
    smem_words = 0
    for i, comp in enumerate(components):
        c = ch.comp[slot]
        comp.pack(c, binder)
        smem_words = _smem_tally(comp, c, smem_words)
        if slot > 0:
            if offsets is None:
                off, rot = np.zeros(3), eye
            else:
                off = np.asarray(offsets[i - 1], dtype=float)
                rot = np.asarray(rotmats[i - 1], dtype=float)
            transform(slot, off, rot)
        if extra[i]:
            slots = [ch.comp[slot + 1 + j] for j in range(extra[i])]
            comp.pack_extra(c, slots, binder)
            for j in range(extra[i]):
                transform(slot + 1 + j, np.zeros(3), eye)
        slot += 1 + extra[i]
    ch.weight_exp2 = weight_exp2(components)
    return ch


def _smem_tally(comp, c, words):
    """Give a monitor a shared-memory tally copy (MCV_COMP_SMEM_TALLY) at
    offset `words` of the block's tally area when it asks for one
    (smem_tally True) or is small (None and at most SMEM_TALLY_AUTO_BINS
    bins) and it fits; returns the area's new size."""
    want = getattr(comp, "smem_tally", False)
    if want is False or not c.tally:
        return words
    nb = comp.nbins()
    if want is None and nb > comp.SMEM_TALLY_AUTO_BINS:
        return words
    if words + 3 * nb > nat.MCV_SMEM_TALLY_MAX:
        if want:
            raise ValueError(f"{comp.name}: {nb} bins do not fit the "
                             "shared-memory tally area")
        return words
    c.flags |= nat.FLAG_SMEM_TALLY
    c.ip[6] = words
    return words + 3 * nb


# where the FP32 kernels place a source's nominal weight: 2^64 leaves 64
# binary orders for weights to grow and 126 + 23 + 64 to shrink before a
# float underflows
WEIGHT_TARGET_EXP2 = 64


def weight_exp2(components):
    """The power of two the FP32 kernels multiply every weight by
    (mcv_chain.weight_exp2): it brings the first component's nominal weight
    (a source's weight on its central ray) to about 2^64.  0 when the chain
    does not start with a source that states one."""
    first = components[0] if components else None
    nominal = getattr(first, "nominal_weight", None)
    w = nominal() if callable(nominal) else None
    if not w or not np.isfinite(w) or w <= 0:
        return 0
    e = int(round(WEIGHT_TARGET_EXP2 - np.log2(w)))
    return max(-100, min(100, e))


def chain_parts(instrument):
    """(components, offsets, rotmats, first) of the chain that runs an
    instrument.  Arms ahead of the first other component are left out:
    the reference runs them as no-ops on a neutron that no source has set
    yet (its generated kernel calls every component in turn,
    acc/run_script.py:58-80), while the engine ends a neutron once its
    weight is not positive, which would end every neutron there.  Frames
    are absolute, so leaving them out changes no transform of the others.
    `first` is the instrument index of chain component 0."""
    offsets, rotmats = calcTransformations(instrument)
    comps = list(instrument.components)
    for comp in comps:
        # components whose physics depends on their orientation in the
        # instrument (gravity in the guide's frame)
        if hasattr(comp, "orient"):
            comp.orient(instrument.geometer.rotation(comp))
    k = 0
    while k < len(comps) - 1 and getattr(comps[k], "opcode", None) == nat.OP_ARM:
        k += 1
    return comps[k:], offsets[k:], rotmats[k:], k


def chain_for_instrument(instrument, binder=None):
    """The chain of an instrument's components (chain_parts) with the frame
    transforms between them.  chain.first_component is the instrument
    index of chain component 0 (the engine's component indices, such as
    replay's `last`, count from it)."""
    comps, offsets, rotmats, k = chain_parts(instrument)
    ch = build_chain(comps, offsets, rotmats, binder)
    ch.first_component = k
    return ch


VARIANTS = {None: 0, "auto": 0, "thread": 1, "regen": 2,
            "regen_noqueue": 3, "fp64_fma": nat.MCV_VARIANT_FP64_FMA}


def _launch(threads_per_block=None, blocks=None, variant=None):
    if not threads_per_block and not blocks and not VARIANTS[variant]:
        return None
    L = nat.mcv_launch()
    L.threads_per_block = int(threads_per_block or 0)
    L.blocks = int(blocks or 0)
    L.variant = VARIANTS[variant]
    return L


def _precision(floattype):
    return config.precision_bits(floattype)


def run_chain(chain, ncount, seed=None, floattype=None, first=0,
              threads_per_block=None, blocks=None, sync=True, device=None,
              variant=None):
    """mcv_run_chain: ncount neutrons through the fused chain kernel
    (variant None/"auto", "thread" or "regen" for FP32; "fp64_fma" for the
    FP64 kernel with contracted multiply-adds).  Returns the mcv_status
    (sync=True) or None."""
    ctx = nat.context(device)
    st = nat.mcv_status() if sync else None
    L = _launch(threads_per_block, blocks, variant)
    seed = config.rng_seed if seed is None else seed
    rc = nat.lib().mcv_run_chain(
        ctx.handle, ctypes.byref(chain), int(ncount), int(first), int(seed),
        _precision(floattype), ctypes.byref(L) if L else None,
        nat.current_stream_handle(), ctypes.byref(st) if st else None)
    nat.check(rc, st)
    return st


def run_instrument(instrument, ncount, **kw):
    chain = chain_for_instrument(instrument)
    return run_chain(chain, ncount, **kw)


def run_components(components, ncount, threads_per_block=None, **kw):
    chain = build_chain(list(components))
    return run_chain(chain, ncount, threads_per_block=threads_per_block, **kw)


def replay(chain, ncount, uniforms=None, seed=None, floattype=None, first=0,
           record=True, threads_per_block=None, blocks=None, device=None):
    """mcv_replay_uniforms: returns (neutrons (ncount, 10) float64 on the
    GPU, last component index (ncount,) int32)."""
    import torch
    ctx = nat.context(device)
    dev = torch.device("cuda", ctx.device)
    st = nat.mcv_status()
    out = torch.empty((int(ncount), 10), dtype=torch.float64, device=dev) \
        if record else None
    last = torch.empty(int(ncount), dtype=torch.int32, device=dev) \
        if record else None
    stride = 0
    uptr = None
    if uniforms is not None:
        u = torch.as_tensor(uniforms, dtype=torch.float32).to(dev).contiguous()
        if u.ndim != 2 or u.shape[0] != ncount:
            raise ValueError("uniforms must have shape (ncount, stride)")
        stride = u.shape[1]
        uptr = ctypes.c_void_p(u.data_ptr())
    L = _launch(threads_per_block, blocks)
    seed = config.rng_seed if seed is None else seed
    rc = nat.lib().mcv_replay_uniforms(
        ctx.handle, ctypes.byref(chain), int(ncount), int(first), int(seed),
        _precision(floattype), uptr, int(stride),
        ctypes.c_void_p(out.data_ptr()) if record else None,
        ctypes.c_void_p(last.data_ptr()) if record else None,
        ctypes.byref(L) if L else None, nat.current_stream_handle(),
        ctypes.byref(st))
    nat.check(rc, st)
    return out, last


def process_buffer(components, neutrons, seed=None, first=0, floattype=None,
                   offsets=None, rotmats=None, device=None):
    """mcv_process_buffer on a host (N, 10) array; returns the updated host
    array (float64)."""
    import torch
    ctx = nat.context(device)
    dev = torch.device("cuda", ctx.device)
    prec = _precision(floattype)
    dt = torch.float32 if prec == 32 else torch.float64
    arr = np.ascontiguousarray(neutrons, dtype=np.float64).reshape(-1, 10)
    buf = torch.from_numpy(arr).to(dev, dtype=dt).contiguous()
    chain = build_chain(list(components), offsets, rotmats)
    st = nat.mcv_status()
    seed = config.rng_seed if seed is None else seed
    rc = nat.lib().mcv_process_buffer(
        ctx.handle, ctypes.byref(chain), ctypes.c_void_p(buf.data_ptr()),
        arr.shape[0], int(first), int(seed), prec, None,
        nat.current_stream_handle(), ctypes.byref(st))
    nat.check(rc, st)
    return buf.to(torch.float64).cpu().numpy()


def intersect(hss_component, rays, floattype="float64", device=None):
    """mcv_intersect: sorted hit times (N, 10; NaN padded) and counts (N,)."""
    import torch
    ctx = nat.context(device)
    dev = torch.device("cuda", ctx.device)
    from .memory import DeviceBinder
    c = hss_component.to_struct(DeviceBinder())
    r = torch.as_tensor(np.asarray(rays, dtype=np.float64).reshape(-1, 6),
                        device=dev).contiguous()
    n = r.shape[0]
    ts = torch.empty((n, nat.MCV_MAX_INTERSECTIONS), dtype=torch.float64,
                     device=dev)
    cnt = torch.empty(n, dtype=torch.int32, device=dev)
    st = nat.mcv_status()
    rc = nat.lib().mcv_intersect(
        ctx.handle, ctypes.byref(c), ctypes.c_void_p(r.data_ptr()), n,
        ctypes.c_void_p(ts.data_ptr()), ctypes.c_void_p(cnt.data_ptr()),
        _precision(floattype), nat.current_stream_handle(), ctypes.byref(st))
    nat.check(rc, st)
    return ts.cpu().numpy(), cnt.cpu().numpy()


def read_status(expected=0, device=None):
    """mcv_ctx_status: synchronise, read and reset the context's counters,
    check `expected` processed neutrons (0 = no check)."""
    ctx = nat.context(device)
    st = nat.mcv_status()
    rc = nat.lib().mcv_ctx_status(ctx.handle, nat.current_stream_handle(),
                                  int(expected), ctypes.byref(st))
    nat.check(rc, st)
    return st


def probe_fma_peak(precision=32, repeats=3, device=None):
    """Measured FMA-pipe peak of the current GPU in TFLOP/s."""
    ctx = nat.context(device)
    out = ctypes.c_double()
    nat.check(nat.lib().mcv_probe_fma_peak(ctx.device, int(precision),
                                           int(repeats), ctypes.byref(out)))
    return out.value


def probe_sfu_rate(repeats=3, device=None):
    """Measured special-function-unit rate of the current GPU (FP32
    base-2 exponentials per second)."""
    ctx = nat.context(device)
    out = ctypes.c_double()
    nat.check(nat.lib().mcv_probe_sfu_rate(ctx.device, int(repeats),
                                           ctypes.byref(out)))
    return out.value


def probe_atomic_rate(nbins, repeats=3, device=None):
    """Measured FP64 atomicAdd rate (ops/s) into `nbins` doubles."""
    ctx = nat.context(device)
    out = ctypes.c_double()
    nat.check(nat.lib().mcv_probe_atomic_rate(ctx.device, int(nbins),
                                              int(repeats), ctypes.byref(out)))
    return out.value


# ------------------------------------------------------------ batched runs
def _batch_arrays(chains, counts, seeds):
    n = len(chains)
    if not 1 <= n <= nat.MCV_MAX_VARIANTS:
        raise ValueError(f"1..{nat.MCV_MAX_VARIANTS} variants, got {n}")
    if len(counts) != n or len(seeds) != n:
        raise ValueError("one count and one seed per variant")
    arr = (nat.mcv_chain * n)()
    for v, ch in enumerate(chains):
        arr[v] = ch
    cnt = (ctypes.c_uint64 * n)(*[int(c) for c in counts])
    sd = (ctypes.c_uint64 * n)(*[int(s) for s in seeds])
    return arr, cnt, sd


def _launch3(threads_per_block=None, blocks=None, chunk=None):
    if not (threads_per_block or blocks or chunk):
        return None
    L = nat.mcv_launch()
    L.threads_per_block = int(threads_per_block or 0)
    L.blocks = int(blocks or 0)
    L.chunk = int(chunk or 0)
    return L


def run_batched(instruments, counts, seeds, floattype=None,
                threads_per_block=None, blocks=None, chunk=None, sync=True,
                device=None):
    """mcv_run_batched: every instrument (variant) runs counts[v] neutrons
    of its own stream seeds[v] in one persistent launch."""
    ctx = nat.context(device)
    chains = [chain_for_instrument(ins) for ins in instruments]
    arr, cnt, sd = _batch_arrays(chains, counts, seeds)
    L = _launch3(threads_per_block, blocks, chunk)
    st = nat.mcv_status() if sync else None
    rc = nat.lib().mcv_run_batched(
        ctx.handle, arr, len(chains), cnt, sd, _precision(floattype),
        ctypes.byref(L) if L else None, nat.current_stream_handle(),
        ctypes.byref(st) if st else None)
    nat.check(rc, st)
    return st


class BatchedGraph:
    """The batched launch captured once in a CUDA graph; `launch()` replays
    it on the current stream (mcv_graph_create_batched / mcv_graph_launch)."""

    def __init__(self, instruments, counts, seeds, floattype=None,
                 threads_per_block=None, blocks=None, chunk=None,
                 device=None):
        self.ctx = nat.context(device)
        self.instruments = list(instruments)
        self.total = int(sum(int(c) for c in counts))
        chains = [chain_for_instrument(ins) for ins in self.instruments]
        arr, cnt, sd = _batch_arrays(chains, counts, seeds)
        L = _launch3(threads_per_block, blocks, chunk)
        self.handle = ctypes.c_void_p()
        rc = nat.lib().mcv_graph_create_batched(
            self.ctx.handle, arr, len(chains), cnt, sd, _precision(floattype),
            ctypes.byref(L) if L else None, ctypes.byref(self.handle))
        nat.check(rc)

    def launch(self):
        nat.check(nat.lib().mcv_graph_launch(self.handle,
                                             nat.current_stream_handle()))

    def close(self):
        if self.handle:
            nat.lib().mcv_graph_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ gradients
def backward(chain, ncount, dout, dparam=None, dtable=None, seed=None,
             floattype=None, first=0, threads_per_block=None, device=None,
             variant=None):
    """mcv_backward: replay `ncount` neutrons of `seed` and add the gradient
    of L into the given device tensors.  dout {component index: float64
    tensor (nbins,) = dL/d(sum p)}, dparam {index: float64 tensor (3,) for a
    guide (m, alpha, W) or (2,) for the sample (mu, sigma)}, dtable {index:
    float64 tensor (S(Q,E) nodes or powder peaks)}.  `variant` as for
    run_chain (the FP32 replay has the forward's kernel structures)."""
    ctx = nat.context(device)
    g = nat.mcv_grad()
    keep = []
    for field, d in (("dout", dout), ("dparam", dparam or {}),
                     ("dtable", dtable or {})):
        arr = getattr(g, field)
        for k, t in d.items():
            if t.dtype.itemsize != 8 or not t.is_cuda or not t.is_contiguous():
                raise ValueError(f"{field}[{k}] must be a contiguous CUDA "
                                 "float64 tensor")
            arr[k] = t.data_ptr()
            keep.append(t)
    st = nat.mcv_status()
    L = _launch(threads_per_block, None, variant)
    seed = config.rng_seed if seed is None else seed
    rc = nat.lib().mcv_backward(
        ctx.handle, ctypes.byref(chain), ctypes.byref(g), int(ncount),
        int(first), int(seed), _precision(floattype),
        ctypes.byref(L) if L else None, nat.current_stream_handle(),
        ctypes.byref(st))
    nat.check(rc, st)
    return st
