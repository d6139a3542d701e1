"""Monitor base (acc/components/monitors/MonitorBase.py:4-12).

A monitor owns a float64 tally of shape (3, *hist_shape) holding
(N, sum p, sum p^2) per bin -- the reference's `out` array
(psd_monitor.py:61-65).  On the GPU it lives in device memory and
accumulates across runs; `out` returns a host copy.
"""

import os

import numpy as np

from ..ComponentBase import ComponentBase
from ... import _native as nat


class Histogram:
    """What getHistogram returns: axes (name, centers, unit), data (I) and
    errors (squared errors), as the `histogram` package's objects carry."""

    def __init__(self, name, axes, data, errors):
        self.name = name
        self.axes = axes
        self.data = self.I = np.asarray(data)
        self.errors = self.E2 = np.asarray(errors)

    def __getattr__(self, key):
        for n, c, _ in self.__dict__.get("axes", ()):
            if n == key:
                return c
        raise AttributeError(key)

    def __truediv__(self, other):
        od = other.data if isinstance(other, Histogram) else other
        return Histogram(self.name, self.axes, self.data / od,
                         self.errors / (od * od))


class MonitorBase(ComponentBase):
    filename = None
    hist_shape = ()
    # warp-aggregated tally atomics (MCV_COMP_AGGREGATE); plain atomics
    # measured faster on GB300 for the bench workloads
    aggregate_tallies = False
    # a per-block copy of the tally in shared memory in the FP32
    # path-regeneration kernel (MCV_COMP_SMEM_TALLY): True, False, or None
    # for monitors of at most SMEM_TALLY_AUTO_BINS bins.  Off by default:
    # on the guide chain (2% of the neutrons reach the monitors) the
    # 200-bin energy monitor's copy measured 1.9% slower on GB300 than its
    # global atomics (shared-memory FP64 atomics, the zeroing and the flush
    # cost more than the L2 atomics they save)
    smem_tally = False
    SMEM_TALLY_AUTO_BINS = 256

    def nbins(self):
        return int(np.prod(self.hist_shape))

    def pack_tally(self, c, binder):
        c.tally = binder.tally(self, self.nbins())
        if self.aggregate_tallies:
            c.flags |= nat.FLAG_AGGREGATE

    @property
    def out(self):
        t = getattr(self, "_device_tally", None)
        if t is None:
            return np.zeros((3,) + tuple(self.hist_shape))
        return t.detach().cpu().numpy().reshape((3,) + tuple(self.hist_shape))

    @property
    def out_N(self):
        return self.out[0]

    @property
    def out_p(self):
        return self.out[1]

    @property
    def out_p2(self):
        return self.out[2]

    def reset(self):
        t = getattr(self, "_device_tally", None)
        if t is not None:
            t.zero_()

    def axes(self):
        raise NotImplementedError

    def histogram_name(self):
        return self.name

    def getHistogram(self, scale_factor=1.):
        out = self.out
        return Histogram(self.histogram_name(), self.axes(),
                         data=out[1] * scale_factor,
                         errors=out[2] * scale_factor * scale_factor)

    def save(self, scale_factor=1.):
        """Write the histogram next to `filename`: HDF5 when h5py is
        installed, otherwise NumPy .npz (MonitorBase.save, :8-12, writes
        HDF5 through the external `histogram` package)."""
        h = self.getHistogram(scale_factor=scale_factor)
        fn = self.filename or (self.name + ".h5")
        try:
            import h5py
        except ImportError:
            h5py = None
        if h5py is not None:
            with h5py.File(fn, "w") as f:
                g = f.create_group(h.name)
                g["data"] = h.data
                g["errors"] = h.errors
                for n, c, u in h.axes:
                    g[f"axis_{n}"] = c
                    g[f"axis_{n}"].attrs["unit"] = u
            return fn
        base, _ = os.path.splitext(fn)
        kw = {f"axis_{n}": c for n, c, _ in h.axes}
        np.savez(base + ".npz", data=h.data, errors=h.errors, **kw)
        return base + ".npz"


def centers(lo, hi, n):
    d = (hi - lo) / n
    return np.arange(lo + d / 2, hi, d)[:n]
