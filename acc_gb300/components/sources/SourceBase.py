"""Source base (acc/components/sources/SourceBase.py:20-59)."""

from ..StochasticComponentBase import StochasticComponentBase


class SourceBase(StochasticComponentBase):

    def process_no_buffer(self, N, threads_per_block=None, ntotalthreads=None):
        """Generate N neutrons with this source alone on the GPU
        (SourceBase.process_no_buffer, :22-34); returns the engine status."""
        from ...engine import run_components
        return run_components([self], int(N), threads_per_block=threads_per_block)
