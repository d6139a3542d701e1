"""Component base classes: the plugin contract of
acc/components/ComponentBase.py:41-137.

A component keeps the reference's constructor signature and its
`propagate_params` tuple (same order and meaning), and packs itself into an
`mcv_component` C struct (`pack`).  The per-neutron `propagate` of each
component is device code inside libacc_gb300.so, selected by the struct's
opcode; `process(neutrons)` runs the component over a neutron array on the
GPU, the buffered mode of ComponentBase.process (:79-107).
"""

import numpy as np

from .. import _native as nat
from .. import config


class Curator(type):
    """Registers concrete component classes (ComponentBase.py:21-32)."""

    components = []

    def __new__(cls, name, bases, dct):
        x = super().__new__(cls, name, bases, dct)
        if not name.endswith("Base"):
            Curator.components.append(x)
        return x


def change_floattype(newtype):
    """Select the working precision of the engine ("float32"/"float64"),
    the global switch of ComponentBase.change_floattype (:34-39)."""
    config.precision_bits(newtype)
    config.floattype = newtype
    ComponentBase._floattype = newtype


def _set(c, k, v):
    c.dp[k] = float(v)
    c.fp[k] = float(v)


class ComponentBase(metaclass=Curator):
    opcode = nat.OP_ARM
    is_multiplescattering = False
    NUM_MULTIPLE_SCATTER = 10
    propagate_params = ()
    _floattype = "float64"

    def __init__(self, name="component", **kwargs):
        self.name = name

    # --------------------------------------------------------- packing
    def pack(self, c, binder):
        """Fill the mcv_component `c` (zeroed) for this component."""
        c.opcode = self.opcode

    def to_struct(self, binder):
        c = nat.mcv_component()
        self.pack(c, binder)
        return c

    # legacy name used by reference callers for the device function; the
    # device code lives in the engine library, selected by `opcode`
    @property
    def propagate(self):
        raise AttributeError(
            f"{type(self).__name__}.propagate is device code in "
            "libacc_gb300.so; run it with process() or run_script.run()")

    @property
    def floattype(self):
        return config.floattype

    def get_numpy_floattype(self):
        return config.get_numpy_floattype()

    # --------------------------------------------------- buffered mode
    def process(self, neutrons, seed=None, first=0):
        """Run this component over `neutrons` ((N, 10) array-like) on the GPU
        and return the survivors (weight > 0), as ComponentBase.process does
        (ComponentBase.py:79-107)."""
        from ..engine import process_buffer
        arr = np.asarray(_as_array(neutrons), dtype=np.float64).reshape(-1, 10)
        out = process_buffer([self], arr, seed=seed, first=first)
        return out[out[:, 9] > 0]


def _as_array(neutrons):
    # an mcni neutron_buffer, when mcni is installed
    if hasattr(neutrons, "__len__") and not isinstance(neutrons, np.ndarray):
        try:
            from mcni.neutron_storage import neutrons_as_npyarr
            a = neutrons_as_npyarr(neutrons)
            return a.reshape(-1, 10)
        except Exception:
            pass
    return neutrons


set_param = _set
