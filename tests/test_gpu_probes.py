"""The measurement probes (include/acc_gb300_probe.h) on the GPU: each
returns a rate inside a plausible range for a GB300 (152 SMs at up to
2.07 GHz): FP32 FMA at most 128 lanes an SM a clock (80.5 TFLOP/s), FP64
FMA far below it, the special-function unit below 64 operations an SM a
clock (2.0e13/s), and FP64 atomics between 1e9 and 1e12 a second."""

import pytest

from acc_gb300 import engine

pytestmark = pytest.mark.gpu


def test_fma_peaks(engine_lib):
    f32 = engine.probe_fma_peak(32, repeats=2)
    f64 = engine.probe_fma_peak(64, repeats=2)
    assert 20.0 < f32 < 81.0, f32
    assert 0.05 < f64 < 0.25 * f32, f64


def test_sfu_rate(engine_lib):
    r = engine.probe_sfu_rate(repeats=2)
    assert 1e12 < r < 2.1e13, r


def test_atomic_rate(engine_lib):
    r = engine.probe_atomic_rate(1 << 24, repeats=2)
    assert 1e9 < r < 1e12, r
