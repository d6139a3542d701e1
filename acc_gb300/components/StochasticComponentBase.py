"""Base of components that draw random numbers
(acc/components/StochasticComponentBase.py:19-64).  The engine gives every
neutron its own Philox stream, so no per-thread RNG state is created."""

from .ComponentBase import ComponentBase


class StochasticComponentBase(ComponentBase):
    pass
