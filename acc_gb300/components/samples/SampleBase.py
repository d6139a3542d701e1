"""Sample base (acc/components/samples/SampleBase.py:16-61)."""

from ..ComponentBase import set_param
from ..StochasticComponentBase import StochasticComponentBase


class SampleBase(StochasticComponentBase):

    def extra_slots(self):
        """Chain slots after this component: a composite kernel's elements
        (include/acc_gb300.h, COMPOSITE)."""
        kernel = getattr(self, "kernel", None)
        return getattr(kernel, "n_slots", 0)

    def pack_extra(self, c, slots, binder):
        self.kernel.pack_elements(c, slots, binder, set_param)
