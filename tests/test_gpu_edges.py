"""Edge cases of the launch and the chain, GPU against the oracle:
no neutrons, neutron counts that fill no block or warp, index ranges that
cross the Philox counter's 32-bit word, and a chain of the maximum length.
FP64 bound as everywhere: 1e-12 relative (denominator floored at the
slot's RMS), identical exit components."""

import numpy as np
import pytest

from acc_gb300 import _native as nat
from acc_gb300 import engine, instruments
from acc_gb300.components.monitors.psd_monitor import PSD_monitor
from acc_gb300.components.optics.arm import Arm
from acc_gb300.components.sources.source_simple import Source_simple
from acc_gb300.instrument import instrument
from helpers import gpu_tallies, oracle_run, rel_err

pytestmark = pytest.mark.gpu


def _record(ins, n, seed, floattype, first=0):
    ch = engine.chain_for_instrument(ins)
    out, last = engine.replay(ch, n, seed=seed, floattype=floattype,
                              first=first)
    return out.cpu().numpy(), last.cpu().numpy()


def _fp64_matches_oracle(builder, n, seed, first=0):
    g_out, g_last = _record(builder(), n, seed, "float64", first)
    _, stats, o_out, o_last = oracle_run(builder(), n, seed=seed,
                                         first=first, record=True)
    assert stats["processed"] == n
    np.testing.assert_array_equal(g_last, o_last)
    assert rel_err(g_out, o_out).max() <= 1e-12


@pytest.mark.parametrize("floattype,variant", [
    ("float64", None), ("float32", "thread"), ("float32", "regen")])
def test_zero_neutrons_touch_nothing(floattype, variant):
    ins = instruments.guide_chain()
    st = engine.run_instrument(ins, 0, seed=1, floattype=floattype,
                               variant=variant)
    assert st.processed == 0
    for t in gpu_tallies(ins).values():
        assert not t.any()


@pytest.mark.parametrize("n", [1, 31, 33, 257, 4099])
def test_ragged_counts(n):
    """FP64 same stream against the oracle; FP32 thread and regeneration
    kernels process exactly n neutrons and count the same entries."""
    _fp64_matches_oracle(instruments.guide_chain, n, seed=3)
    a, b = instruments.guide_chain(), instruments.guide_chain()
    sa = engine.run_instrument(a, n, seed=3, floattype="float32",
                               variant="regen")
    sb = engine.run_instrument(b, n, seed=3, floattype="float32",
                               variant="thread")
    assert sa.processed == sb.processed == n
    for ta, tb in zip(gpu_tallies(a).values(), gpu_tallies(b).values()):
        assert ta[0].sum() == tb[0].sum()


def test_index_range_across_the_counter_word():
    """Neutron indices 2^32 - 9 .. 2^32 + 10: the counter's high word
    changes inside the range; the GPU draws what the oracle draws."""
    _fp64_matches_oracle(instruments.sphere_theta_tof, 20, seed=5,
                         first=2 ** 32 - 9)


def _longest_chain():
    """A source, 30 arms at turned and shifted frames, and a PSD monitor:
    MCV_MAX_COMPONENTS components, each hop a full frame transform."""
    ins = instrument("longest_chain")
    ins.append(Source_simple("source", radius=0.01, dist=3.1, xw=0.02,
                             yh=0.02, E0=60.0, dE=10.0), position=(0, 0, 0))
    for i in range(nat.MCV_MAX_COMPONENTS - 2):
        ins.append(Arm(f"arm{i}"), position=(0.001 * (i % 3), 0, 0.1 * i),
                   orientation=(0, 2.0 * ((i % 5) - 2), 1.0 * (i % 2)))
    ins.append(PSD_monitor("psd", xmin=-0.03, xmax=0.03, ymin=-0.03,
                           ymax=0.03, nx=50, ny=50, filename="psd.h5"),
               position=(0, 0, 3.1))
    return ins


def test_chain_of_maximum_length():
    ins = _longest_chain()
    assert engine.chain_for_instrument(ins).ncomp == nat.MCV_MAX_COMPONENTS
    _fp64_matches_oracle(_longest_chain, 5000, seed=9)
    a = _longest_chain()
    engine.run_instrument(a, 200000, seed=9, floattype="float32")
    b = _longest_chain()
    engine.run_instrument(b, 200000, seed=9, floattype="float64")
    ta, tb = a.components[-1].out, b.components[-1].out
    assert ta[0].sum() > 1000
    # the same stream: entries move only where a hit lies within float
    # rounding of a bin edge
    assert np.abs(ta[0] - tb[0]).sum() / 2 <= 1e-3 * tb[0].sum()
