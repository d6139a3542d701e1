"""Global run settings (the module globals of acc/config.py:1-4).

`threads_per_block` above the engine's 256-thread launch bound is clamped;
`ntotalthreads` is accepted for compatibility (the engine sizes its grid
from the SM count and strides over neutrons, so the value does not change
results).  `floattype` selects the FP64 plain kernels ("float64", the
reference's default) or the fused FP32 kernels ("float32").
"""

ntotalthreads = int(1e6)
threads_per_block = 512
floattype = "float64"
rng_seed = 1


def get_numpy_floattype():
    import numpy as np
    return getattr(np, floattype)


def precision_bits(ft=None):
    ft = ft or floattype
    if ft in ("float32", "f32", 32):
        return 32
    if ft in ("float64", "f64", 64):
        return 64
    raise ValueError(f"unknown float type {ft!r}")
