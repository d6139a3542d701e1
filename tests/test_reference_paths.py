"""Per-component parity against outputs of the reference's own code.

``tests/golden/reference_paths.npz`` holds, for each case of
``tests/golden/reference_cases.py``, input neutrons, float32 uniforms and
the neutrons (and monitor histograms) that the reference's device
functions produced from them, run as Python on the CPU by
``tests/golden/make_reference_fixtures.py``.  Here the same component of
this package runs on the same inputs with the same uniforms injected:

* the oracle (CPU): every slot within 1e-12 relative (denominator floored
  at the slot's RMS over the batch), histogram counts exact and sums
  within 1e-12;
* the GPU engine, FP64: the same bounds;
* the GPU engine, FP32: every slot of at least 99.5% of the neutrons
  within 1e-5 relative, none beyond 1e-3 unless it crossed a branch
  (a neutron absorbed in one run and not in the other, at most 1%), and
  histogram counts within 1% of the entries moved between bins (float
  rounding at a bin edge).  The SNS and STS sources draw E and t in FP32
  from inverse tables, t by sampling the two-row mixture the reference
  inverts, so their E and t are other (equally distributed) draws from the
  same uniforms: there the position and the flight direction are held to
  the bound, and E and t to their distributions (test_gpu_parity.py).
"""

import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_cases as RC  # noqa: E402
from helpers import gpu_tallies, oracle_run, rel_err  # noqa: E402

FIXTURE = os.path.join(HERE, "golden", "reference_paths.npz")
DATA = np.load(FIXTURE)
META = json.load(open(os.path.join(HERE, "golden", "reference_paths.json")))
NAMES = list(RC.CASES)


def _case(name):
    inp = DATA[name + ".in"] if name + ".in" in DATA else None
    return (inp, DATA[name + ".u"], DATA[name + ".out"],
            DATA[name + ".valid"], DATA.get(name + ".hist"))


def _is_monitor(name):
    return RC.CASES[name]["kind"].endswith("monitor") or \
        RC.CASES[name]["kind"] == "psd_monitor_4pi"


def test_fixture_covers_every_case():
    for name in NAMES:
        inp, u, out, valid, hist = _case(name)
        assert valid.all(), name
        assert out.shape == (RC.CASES[name]["n"], 10)
        assert (META[name]["max_uniforms"] <= u.shape[1])
    # the reference takes one float32 square root of a uniform (the disc
    # source's radius, source_simple.py:139); nothing else
    assert META["_float32_math"] == ["sqrt"]


def test_fixture_inputs_are_the_seeded_draws():
    for ci, name in enumerate(NAMES):
        inp, u, _, _, _ = _case(name)
        np.testing.assert_array_equal(u, RC.draw_uniforms(RC.CASES[name],
                                                          100 + ci))
        ref = RC.draw_inputs(RC.CASES[name], 100 + ci)
        if ref is None:
            assert inp is None
        else:
            np.testing.assert_array_equal(inp, ref)


def _check_fp64(name, out, hist, got, got_hist):
    _, _, ref, valid, _ = _case(name)
    err = rel_err(got[valid], ref[valid])
    assert err.max() <= 1e-12, (name, err.max(), np.unravel_index(
        err.argmax(), err.shape))
    if hist is not None:
        np.testing.assert_array_equal(got_hist[0], hist[0])
        np.testing.assert_allclose(got_hist[1:], hist[1:], rtol=1e-12,
                                   atol=1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name):
    inp, u, ref, valid, hist = _case(name)
    ins = RC.product_instrument(name, inp)
    tallies, stats, out, last = oracle_run(ins, len(u), uniforms=u,
                                           record=True)
    got_hist = None
    if hist is not None:
        (c, got_hist), = tallies.items()
        got_hist = got_hist.reshape(hist.shape)
    _check_fp64(name, out, hist, out, got_hist)


def _gpu_run(name, floattype):
    from acc_gb300 import engine
    inp, u, ref, valid, hist = _case(name)
    ins = RC.product_instrument(name, inp)
    ch = engine.chain_for_instrument(ins)
    out, last = engine.replay(ch, len(u), uniforms=u, seed=1,
                              floattype=floattype)
    got_hist = None
    if hist is not None:
        (_, got_hist), = gpu_tallies(ins).items()
        got_hist = np.asarray(got_hist).reshape(hist.shape)
    return out.cpu().numpy(), got_hist


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp64_matches_reference(name, engine_lib):
    _, _, _, _, hist = _case(name)
    out, got_hist = _gpu_run(name, "float64")
    _check_fp64(name, out, hist, out, got_hist)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp32_matches_reference(name, engine_lib):
    _, _, ref, valid, hist = _case(name)
    out, got_hist = _gpu_run(name, "float32")
    ref, out = ref[valid], out[valid]
    if RC.CASES[name]["kind"] in ("sns_source", "sts_source"):
        def pos_dir(a):
            d = a[:, 3:6] / np.linalg.norm(a[:, 3:6], axis=1, keepdims=True)
            return np.concatenate([a[:, :3], d], axis=1)
        err = rel_err(pos_dir(out), pos_dir(ref)).max(axis=1)
        assert (err > 1e-5).mean() <= 0.005, (name, np.sort(err)[-5:])
        return
    alive_r, alive_g = ref[:, 9] > 0, out[:, 9] > 0
    flipped = alive_r != alive_g
    assert flipped.mean() <= 0.01, (name, flipped.sum())
    both = alive_r & alive_g
    err = rel_err(out[both], ref[both]).max(axis=1)
    assert (err > 1e-5).mean() <= 0.005, (name, np.sort(err)[-5:])
    assert (err > 1e-3).sum() <= max(1, 0.01 * both.sum()), \
        (name, np.sort(err)[-5:])
    if hist is not None:
        moved = np.abs(got_hist[0] - hist[0]).sum() / 2
        assert moved <= max(1, 0.01 * hist[0].sum()), (name, moved)
        np.testing.assert_allclose(got_hist[1].sum(), hist[1].sum(),
                                   rtol=1e-3)
