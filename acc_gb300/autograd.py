"""Differentiable instrument runs (torch.autograd).

    run = GradRun(instrument, loss_monitor, ncount, seed,
                  params={"S": ("sqe_table", sample),
                          "mu": ("hss_mu", sample)})
    hist = run(S=table_tensor, mu=mu_tensor)     # sum p per detector bin
    loss = ((hist - target) ** 2).sum(); loss.backward()

The forward is the fused kernel (mcv_run_chain); the backward replays the
same neutrons from their Philox counters (mcv_backward) and accumulates
dL/d theta = sum_bins dL/dH_b sum_{n in b} p_n d ln p_n / d theta.  The
parameters supported are the ones that enter only neutron weights:

  "sqe_table"  S(Q,E) nodes of an SQEGridKernel sample (float32 tensor)
  "hss_mu"     absorption coefficient at 2200 m/s of the sample (1/m)
  "hss_sigma"  scattering coefficient of an isotropic / S(Q,E) sample (1/m)
  "powder_F2"  F^2 of each powder peak (SimplePowderDiffractionKernel)
  "guide_m", "guide_alpha", "guide_W"   supermirror coating of one guide
               or of a list of guides sharing the value
"""

import ctypes

import numpy as np
import torch

from . import engine
from .components.monitors.MonitorBase import MonitorBase
from .components.ComponentBase import set_param
from .memory import DeviceBinder

_GUIDE_SLOT = {"guide_m": (8, 0), "guide_alpha": (7, 1), "guide_W": (9, 2)}


class GradRun:
    """`shard` = (rank, world[, group]): this process runs the neutron block
    sharding.shard_range(ncount, rank, world) and the histogram and the
    gradients are summed over the ranks (torch.distributed all-reduce)."""

    def __init__(self, instrument, loss_monitor, ncount, seed=1,
                 floattype="float64", params=None, shard=None):
        from .sharding import shard_range
        self.shard = None
        self.first, self.count = 0, int(ncount)
        if shard is not None:
            rank, world = int(shard[0]), int(shard[1])
            group = shard[2] if len(shard) > 2 else None
            self.shard = (rank, world, group)
            self.first, self.count = shard_range(ncount, rank, world)
        self.ins = instrument
        self.comps, off, rot, _ = engine.chain_parts(instrument)
        self.mon = loss_monitor
        if not isinstance(loss_monitor, MonitorBase):
            raise TypeError("loss_monitor must be a monitor of the instrument")
        self.mon_index = self._index(loss_monitor)
        self.ncount = int(ncount)
        self.seed = int(seed)
        self.floattype = floattype
        self.params = dict(params or {})
        self.binder = DeviceBinder()
        self.chain = engine.build_chain(self.comps, off, rot, self.binder)

    def _index(self, comp):
        for k, c in enumerate(self.comps):
            if c is comp:
                return k
        raise ValueError(f"{comp!r} is not in the instrument")

    # ------------------------------------------------------ parameters
    def _apply(self, values):
        """Write parameter values into the chain description."""
        for name, (kind, target) in self.params.items():
            if name not in values:
                continue
            v = values[name]
            if kind in _GUIDE_SLOT:
                slot = _GUIDE_SLOT[kind][0]
                for g in _as_list(target):
                    set_param(self.chain.comp[self._index(g)], slot, float(v))
            elif kind == "hss_mu":
                set_param(self.chain.comp[self._index(target)], 8, float(v))
            elif kind == "hss_sigma":
                set_param(self.chain.comp[self._index(target)], 9, float(v))
            elif kind == "sqe_table":
                t = v.detach().to(device="cuda", dtype=torch.float32)
                t = t.contiguous()
                c = self.chain.comp[self._index(target)]
                if tuple(t.shape) != (c.ip[4], c.ip[5]):
                    raise ValueError("table shape differs from the kernel's")
                self._keep_table = t
                c.table = c.ftable = t.data_ptr()
            elif kind == "powder_F2":
                ker = target.kernel
                f2 = np.asarray(v.detach().cpu().numpy(), dtype=np.float64)
                pd = ker.pd
                base = pd.my_s_v2 / np.array([p.F_squared for p in ker.peaks])
                s = base * f2
                tab = np.stack([pd.q_v, pd.w_v, s, np.cumsum(s)], axis=1)
                self._keep_powder = (
                    torch.from_numpy(tab).cuda(),
                    torch.from_numpy(tab.astype(np.float32)).cuda())
                c = self.chain.comp[self._index(target)]
                c.table = self._keep_powder[0].data_ptr()
                c.ftable = self._keep_powder[1].data_ptr()
                self._powder_base = base
            else:
                raise ValueError(f"unknown parameter kind {kind!r}")

    # --------------------------------------------------------- passes
    def forward_hist(self, values):
        self._apply(values)
        t = self.mon._device_tally
        t.zero_()
        st = engine.run_chain(self.chain, self.count, seed=self.seed,
                              floattype=self.floattype, first=self.first)
        assert st.processed == self.count
        if self.shard is not None:
            from .sharding import reduce_tallies
            reduce_tallies([t], self.shard[2])
        n = self.mon.nbins()
        return t[n:2 * n].clone().reshape(self.mon.hist_shape)

    def backward_grads(self, values, grad_hist):
        self._apply(values)
        dout = grad_hist.detach().to(torch.float64).contiguous().reshape(-1)
        dparam, dtable, out = {}, {}, {}
        for name, (kind, target) in self.params.items():
            if kind in _GUIDE_SLOT:
                for g in _as_list(target):
                    k = self._index(g)
                    dparam.setdefault(k, torch.zeros(3, dtype=torch.float64,
                                                     device="cuda"))
            elif kind in ("hss_mu", "hss_sigma"):
                k = self._index(target)
                dparam.setdefault(k, torch.zeros(3, dtype=torch.float64,
                                                 device="cuda"))
            elif kind in ("sqe_table", "powder_F2"):
                k = self._index(target)
                c = self.chain.comp[k]
                size = c.ip[4] * c.ip[5] if kind == "sqe_table" else c.ip[4]
                dtable[k] = torch.zeros(size, dtype=torch.float64,
                                        device="cuda")
        engine.backward(self.chain, self.count, {self.mon_index: dout},
                        dparam, dtable, seed=self.seed,
                        floattype=self.floattype, first=self.first)
        for name, (kind, target) in self.params.items():
            if kind in _GUIDE_SLOT:
                j = _GUIDE_SLOT[kind][1]
                out[name] = sum(dparam[self._index(g)][j]
                                for g in _as_list(target))
            elif kind == "hss_mu":
                out[name] = dparam[self._index(target)][0]
            elif kind == "hss_sigma":
                out[name] = dparam[self._index(target)][1]
            elif kind == "sqe_table":
                c = self.chain.comp[self._index(target)]
                out[name] = dtable[self._index(target)].reshape(
                    c.ip[4], c.ip[5])
            elif kind == "powder_F2":
                out[name] = dtable[self._index(target)] * torch.from_numpy(
                    self._powder_base).cuda()
        if self.shard is not None:
            from .sharding import reduce_gradients
            out = {k: (v if isinstance(v, torch.Tensor) else
                       torch.tensor(float(v), dtype=torch.float64,
                                    device="cuda")).clone()
                   for k, v in out.items()}
            reduce_gradients(out, self.shard[2])
        return out

    def __call__(self, **values):
        names = list(values)
        return _RunFn.apply(self, names, *[values[n] for n in names])


def _as_list(x):
    return list(x) if isinstance(x, (list, tuple)) else [x]


class _RunFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, run, names, *tensors):
        ctx.run = run
        ctx.names = names
        ctx.save_for_backward(*tensors)
        return run.forward_hist(dict(zip(names, tensors)))

    @staticmethod
    def backward(ctx, grad_hist):
        tensors = ctx.saved_tensors
        values = dict(zip(ctx.names, tensors))
        g = ctx.run.backward_grads(values, grad_hist)
        out = []
        for n, t in zip(ctx.names, tensors):
            gn = g[n]
            out.append(gn.to(dtype=t.dtype, device=t.device).reshape(t.shape)
                       if isinstance(gn, torch.Tensor)
                       else torch.tensor(float(gn), dtype=t.dtype,
                                         device=t.device))
        return (None, None, *out)
