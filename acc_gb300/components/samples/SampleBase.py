"""Sample base (acc/components/samples/SampleBase.py:16-61)."""

from ..StochasticComponentBase import StochasticComponentBase


class SampleBase(StochasticComponentBase):
    pass
