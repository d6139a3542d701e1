"""Neutrons replayed from storage
(acc/components/sources/neutronfromstorage.py:42-82): neutron i of a run
is stored neutron i mod N."""

import numpy as np

from ... import _native as nat
from .SourceBase import SourceBase

category = 'sources'


def load_neutrons(path):
    """An (N, 10) float64 array [x y z vx vy vz sx sy t p] from `path`: a
    neutron storage file (.mcv, read as neutronfromstorage.py:58-61 reads
    it) or a NumPy .npy array."""
    if str(path).endswith(".npy"):
        return np.load(path)
    from ...neutron_storage import load
    return load(path)


class NeutronFromStorage(SourceBase):
    opcode = nat.OP_NEUTRON_STORAGE
    requires_neutron_index_in_processing = True

    def __init__(self, name, path=None, neutrons=None):
        """`path`: a neutron storage file (.mcv) or an (N, 10) .npy array;
        or `neutrons`, the array itself (x y z vx vy vz sx sy t p a
        row)."""
        self.name = name
        if neutrons is None:
            neutrons = load_neutrons(path)
        neutrons = np.ascontiguousarray(neutrons, dtype=np.float64)
        if neutrons.ndim != 2 or neutrons.shape[1] != 10 or not len(neutrons):
            raise ValueError("stored neutrons must be an (N, 10) array")
        self.propagate_params = (neutrons,)

    def nominal_weight(self):
        """The median positive weight of the stored neutrons."""
        p = self.propagate_params[0][:, 9]
        p = p[p > 0]
        return float(np.median(p)) if len(p) else None

    def pack(self, c, binder):
        (neutrons,) = self.propagate_params
        c.opcode = self.opcode
        flat = neutrons.reshape(-1)
        c.table = binder.table(self, "neutrons", flat, np.float64)
        c.ftable = binder.table(self, "neutrons_f32", flat, np.float32)
        c.table_len = flat.size
