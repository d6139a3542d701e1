"""GB300-native engine for mcvine.acc's per-neutron propagation chain.

The instrument (source, guides, sample, monitors) runs as one fused CUDA
kernel for sm_103a inside libacc_gb300.so, reached through the C ABI of
include/acc_gb300.h.  The Python layer keeps the component classes,
`propagate_params` and `run_script.run` of mcvine.acc.
"""

from .instrument import Instrument, instrument  # noqa: F401

__version__ = "0.1.0"
