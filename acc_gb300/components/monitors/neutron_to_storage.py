"""Neutrons saved to a storage file where they pass: mcvine's
NeutronToStorage monitor, which the reference's instrument factory places
before and after the component under test (acc/test/instrument_factory.py:
104-113) to write `before_<name>.mcv` and `after_<name>.mcv`.

On the GPU the component appends each neutron that reaches it, unchanged
and in its own frame, to a device buffer (include/acc_gb300.h,
NEUTRON_TO_STORAGE): its index in the run, then its 10 values.  Lanes that
arrive together reserve their rows with one atomic, so rows land in no
fixed order; the host sorts them by neutron index (then by value, for the
scattered neutrons of one incident neutron) before writing, so the file is
the same from run to run.  Weights are saved as they are (no 1/ncount).
"""

import numpy as np

from ... import _native as nat
from ...neutron_storage import save as save_neutrons
from ..ComponentBase import ComponentBase

category = 'monitors'

ROW_WORDS = 11


def decode(buffer):
    """(indices (k,) uint64, neutrons (k, 10) float64, reached) of a
    storage buffer: word 0 counts the neutrons that reached the component,
    rows of [index, 10 values] follow; k = min(reached, capacity).  Rows
    come back sorted by index, then by their values."""
    w = np.ascontiguousarray(buffer, dtype=np.float64)
    reached = int(w[:1].view(np.uint64)[0])
    cap = (w.size - 1) // ROW_WORDS
    k = min(reached, cap)
    rows = w[1:1 + ROW_WORDS * k].reshape(k, ROW_WORDS)
    idx = rows.view(np.uint64)[:, 0].copy()
    neutrons = rows[:, 1:]
    order = np.lexsort([neutrons[:, j] for j in range(9, -1, -1)] + [idx])
    return idx[order], np.ascontiguousarray(neutrons[order]), reached


class NeutronToStorage(ComponentBase):
    opcode = nat.OP_NEUTRON_TO_STORAGE
    # run_script saves it with the monitors
    saves_neutrons = True
    DEFAULT_CAPACITY = 1 << 20

    def __init__(self, name, path="neutrons.mcv", append=False,
                 capacity=None):
        """Save the neutrons reaching this point to `path` (a .mcv file;
        `append` adds to an existing one).  `capacity`: rows of device
        memory (88 bytes each); by default room for every neutron of the
        run that run_script starts, else DEFAULT_CAPACITY.  A run in which
        more neutrons arrive (a multiple scatterer upstream fans them out)
        needs a larger capacity: saving then raises."""
        self.name = name
        self.path = path
        self.append = bool(append)
        if capacity is not None and int(capacity) < 1:
            raise ValueError("capacity must be >= 1")
        self.capacity = None if capacity is None else int(capacity)
        self._expected = None
        self.propagate_params = ()

    def expect_neutrons(self, ncount):
        """Room for `ncount` neutrons unless a capacity was given."""
        self._expected = int(ncount)

    def rows(self):
        if self.capacity is not None:
            return self.capacity
        return max(1, self._expected or self.DEFAULT_CAPACITY)

    def pack(self, c, binder):
        c.opcode = self.opcode
        cap = self.rows()
        c.tally = binder.buffer(self, "rows", 1 + ROW_WORDS * cap)
        c.table_len = cap

    def _buffer(self):
        t = getattr(self, "_device_buffers", {}).get("rows")
        return None if t is None else t.detach().cpu().numpy()

    def stored(self, buffer=None):
        """(indices, neutrons, reached) saved so far on the device (or in
        `buffer`, a host binder's)."""
        b = self._buffer() if buffer is None else buffer
        if b is None:
            return (np.zeros(0, np.uint64), np.zeros((0, 10)), 0)
        return decode(b)

    @property
    def neutrons(self):
        return self.stored()[1]

    def reset(self):
        t = getattr(self, "_device_buffers", {}).get("rows")
        if t is not None:
            t.zero_()

    def save(self, scale_factor=1.):
        """Write the saved neutrons to `path` (weights as they are:
        `scale_factor` is the monitors' 1/ncount and does not apply)."""
        idx, neutrons, reached = self.stored()
        if reached > len(neutrons):
            raise RuntimeError(
                f"NeutronToStorage {self.name}: {reached} neutrons reached it "
                f"but it holds {len(neutrons)}; give it capacity >= {reached}")
        save_neutrons(self.path, neutrons, append=self.append)
        return self.path
