"""Where a chain's tallies and lookup tables live.

A component packs raw pointers into its mcv_component.  A binder supplies
them: `DeviceBinder` hands out CUDA memory (torch tensors kept on the
component, so a monitor's tally persists across runs like the reference's
`out` array, psd_monitor.py:61-65), `HostBinder` hands out NumPy memory for
callers of the same C structs on the host.
"""

import numpy as np


class DeviceBinder:
    """CUDA memory owned by the components themselves."""

    kind = "device"

    def __init__(self, device=None):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("a DeviceBinder needs a CUDA device")
        if device is None:
            device = torch.cuda.current_device()
        self.device = torch.device("cuda", device if isinstance(device, int)
                                   else torch.device(device).index or 0)

    def tally(self, comp, nbins):
        import torch
        t = getattr(comp, "_device_tally", None)
        if t is None or t.numel() != 3 * nbins or t.device != self.device:
            t = torch.zeros(3 * nbins, dtype=torch.float64, device=self.device)
            comp._device_tally = t
        return t.data_ptr()

    def buffer(self, comp, key, n):
        """A zeroed float64 device buffer of `n` values, kept on `comp` (a
        component's output that is not a histogram); reused while its size
        holds."""
        import torch
        cache = comp.__dict__.setdefault("_device_buffers", {})
        t = cache.get(key)
        if t is None or t.numel() != n or t.device != self.device:
            t = torch.zeros(int(n), dtype=torch.float64, device=self.device)
            cache[key] = t
        return t.data_ptr()

    def table(self, comp, key, array, dtype):
        import torch
        cache = comp.__dict__.setdefault("_device_tables", {})
        t = cache.get(key)
        if t is None or t.device != self.device:
            a = np.ascontiguousarray(array, dtype=dtype)
            t = torch.from_numpy(a).to(self.device)
            cache[key] = t
        return t.data_ptr()


class HostBinder:
    """NumPy memory held by the binder (one set per binder)."""

    kind = "host"

    def __init__(self):
        self.tallies = {}
        self.buffers = {}
        self._tables = {}

    def buffer(self, comp, key, n):
        k = (id(comp), key)
        a = self.buffers.get(k)
        if a is None or a.size != n:
            a = np.zeros(int(n))
            self.buffers[k] = a
        return a.ctypes.data

    def tally(self, comp, nbins):
        a = self.tallies.get(id(comp))
        if a is None or a.size != 3 * nbins:
            a = np.zeros(3 * nbins)
            self.tallies[id(comp)] = a
        return a.ctypes.data

    def table(self, comp, key, array, dtype):
        k = (id(comp), key)
        a = self._tables.get(k)
        if a is None:
            a = np.ascontiguousarray(array, dtype=dtype)
            self._tables[k] = a
        return a.ctypes.data

    def out(self, comp):
        """The (3, *shape) tally of a monitor, as the reference's `out`."""
        return self.tallies[id(comp)].reshape((3,) + tuple(comp.hist_shape))
