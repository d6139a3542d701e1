"""mcv_run_batched_noalloc (static device scratch, no allocation) against
mcv_run_batched (context-allocated staging), both through the C ABI.

Same variants, counts and seeds on both entry points, two calls in a row;
the second call uses fewer variants and other seeds and counts, so a stale
description, count or counter left in the static scratch would show.
Tolerance: identical bin counts, sums within 1e-12 relative (only the
order of the atomic additions differs).  The file is collected last so
that the static scratch has been through every earlier test's process
state when it runs; it also passes alone.
"""

import ctypes

import numpy as np
import pytest
import torch

from acc_gb300 import _native as nat
from acc_gb300 import engine, instruments


def _variants(n, seed):
    return instruments.sphere_variants(nvariants=n, nmin=2e4, nmax=2e5,
                                       seed=seed)


def _noalloc(insts, counts, seeds, floattype, chunk=None):
    chains = [engine.chain_for_instrument(i) for i in insts]
    arr, cnt, sd = engine._batch_arrays(chains, counts, seeds)
    L = engine._launch3(None, None, chunk)
    st = nat.mcv_status()
    rc = nat.lib().mcv_run_batched_noalloc(
        arr, len(chains), cnt, sd, engine._precision(floattype),
        ctypes.byref(L) if L else None, nat.current_stream_handle(),
        ctypes.byref(st))
    nat.check(rc, st)
    return st


def _same(a, b):
    for x, y in zip(a, b):
        tx, ty = x.components[-1].out, y.components[-1].out
        np.testing.assert_array_equal(tx[0], ty[0])
        np.testing.assert_allclose(tx[1:], ty[1:], rtol=1e-12, atol=1e-300)
        assert tx[0].sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("floattype", ["float64", "float32"])
def test_noalloc_matches_batched_two_calls(engine_lib, floattype):
    torch.cuda.init()
    ours, counts, seeds = _variants(6, seed=11)
    ref, _, _ = _variants(6, seed=11)
    st = _noalloc(ours, counts, seeds, floattype, chunk=3000)
    assert st.processed == sum(counts)
    st_ref = engine.run_batched(ref, counts, seeds, floattype=floattype,
                                chunk=3000)
    assert st_ref.processed == st.processed
    _same(ours, ref)
    # second call in a row: fewer variants, other seeds and counts, into the
    # same tallies (they accumulate on both sides)
    counts2 = [c // 2 + 17 for c in counts[:4]]
    seeds2 = [s + 1000 for s in seeds[:4]]
    st = _noalloc(ours[:4], counts2, seeds2, floattype)
    assert st.processed == sum(counts2)
    engine.run_batched(ref[:4], counts2, seeds2, floattype=floattype)
    _same(ours, ref)


def test_noalloc_rejects_more_variants_than_the_scratch_holds():
    n = nat.MCV_NOALLOC_MAX_VARIANTS + 1
    arr = (nat.mcv_chain * n)()
    cnt = (ctypes.c_uint64 * n)(*([1] * n))
    sd = (ctypes.c_uint64 * n)(*range(n))
    st = nat.mcv_status()
    rc = nat.lib().mcv_run_batched_noalloc(arr, n, cnt, sd, 64, None, None,
                                           ctypes.byref(st))
    assert rc == nat.MCV_ECAPACITY
    assert b"static scratch maximum of 64" in st.message
