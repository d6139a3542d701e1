"""Batched persistent launch, its CUDA-graph capture and the autotuner
(through the C ABI).  Tolerances: FP64, identical bin counts and sums
within 1e-12 relative (only the order of atomic additions differs)."""

import numpy as np
import pytest
import torch

from acc_gb300 import autotune, engine, instruments

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    torch.cuda.init()
    yield


def variants(n=5, seed=4):
    return instruments.sphere_variants(nvariants=n, nmin=1e4, nmax=2e5,
                                       seed=seed)


def tally(ins):
    return ins.components[-1].out


def test_batched_equals_one_run_per_variant():
    ins, counts, seeds = variants()
    st = engine.run_batched(ins, counts, seeds, floattype="float64",
                            chunk=1000)
    assert st.processed == sum(counts)
    ref, _, _ = variants()
    for v, r in enumerate(ref):
        engine.run_instrument(r, counts[v], seed=seeds[v],
                              floattype="float64")
        a, b = tally(ins[v]), tally(r)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_allclose(a[1:], b[1:], rtol=1e-12, atol=1e-300)
        assert a[0].sum() > 0


def test_batched_uneven_counts_and_empty_variant():
    ins, counts, seeds = variants(n=4, seed=9)
    counts[1] = 0
    counts[2] = 1
    st = engine.run_batched(ins, counts, seeds, floattype="float32",
                            chunk=777)
    assert st.processed == sum(counts)
    assert tally(ins[1])[0].sum() == 0


def test_graph_replay_accumulates():
    ins, counts, seeds = variants(n=3, seed=5)
    g = engine.BatchedGraph(ins, counts, seeds, floattype="float32",
                            chunk=4096)
    g.launch()
    st = engine.read_status(expected=sum(counts))
    assert st.processed == sum(counts)
    once = [tally(i).copy() for i in ins]
    g.launch()
    engine.read_status(expected=sum(counts))
    for i, t1 in zip(ins, once):
        t2 = tally(i)
        np.testing.assert_array_equal(t2[0], 2 * t1[0])
        np.testing.assert_allclose(t2[1:], 2 * t1[1:], rtol=1e-12)
    g.close()


def test_autotuner_keeps_tallies(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "cache.json"))
    ins, counts, seeds = variants(n=3, seed=6)
    engine.run_batched(ins, counts, seeds, floattype="float32")
    before = [tally(i).copy() for i in ins]
    best = autotune.tune_batched(ins, counts, seeds, fraction=0.2,
                                 candidates=[(128, 2, 2048), (256, 4, 8192)])
    assert best["threads_per_block"] in (128, 256)
    assert best["chunk"] in (2048, 8192)
    for i, b in zip(ins, before):
        np.testing.assert_array_equal(tally(i), b)
    assert autotune.tune_batched(ins, counts, seeds) == best  # cached
    one = instruments.guide_chain()
    c = autotune.tune_chain(one, 200000, candidates=[(256, 4), (128, 8)])
    assert c["threads_per_block"] in (128, 256)
    assert tally(one)[0].sum() == 0
