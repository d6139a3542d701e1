"""Neutron storage: the .mcv format (pinned on the reference's own fixture
files, tests/golden/mcv), NeutronFromStorage reading it, and the
NeutronToStorage component on the oracle and on the GPU."""

import os

import numpy as np
import pytest

from acc_gb300 import neutron_storage as ns
from acc_gb300.components.monitors.neutron_to_storage import (
    NeutronToStorage, decode)
from acc_gb300.engine import build_chain, chain_for_instrument
from acc_gb300.memory import HostBinder

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "mcv")
# the reference tree, when present (the fixtures' copy check only)
REF_SOURCES = os.path.join(os.environ.get("MCVINE_ACC_REFERENCE", ""),
                           "tests", "components", "sources")

# create_neutron_storage_for_test.py: the neutron each fixture holds
FIXTURES = {
    "singletestneutron.mcv": np.arange(10.0),
    "singletestneutron2.mcv": np.array([0, 0, 0, 0, 0, 1000.0, 0, 0, 0, 1]),
}


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_fixture_read_and_written_byte_for_byte(name, tmp_path):
    path = os.path.join(GOLDEN, name)
    a = ns.load(path)
    assert a.shape == (1, 10)
    np.testing.assert_array_equal(a[0], FIXTURES[name])
    out = tmp_path / name
    ns.save(out, FIXTURES[name])
    assert out.read_bytes() == open(path, "rb").read()


@pytest.mark.skipif(not os.environ.get("MCVINE_ACC_REFERENCE")
                    or not os.path.isdir(REF_SOURCES),
                    reason="MCVINE_ACC_REFERENCE does not name the "
                           "reference tree")
@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_fixture_copies_match_the_reference(name):
    mine = open(os.path.join(GOLDEN, name), "rb").read()
    assert mine == open(os.path.join(REF_SOURCES, name), "rb").read()


def test_append_wrap_and_partial_reads(tmp_path):
    rng = np.random.default_rng(3)
    a, b = rng.normal(size=(7, 10)), rng.normal(size=(5, 10))
    p = tmp_path / "n.mcv"
    ns.save(p, a)
    ns.save(p, b, append=True)
    assert os.path.getsize(p) == ns.HEADER_BYTES + 12 * 80
    np.testing.assert_array_equal(ns.load(p), np.vstack([a, b]))
    with ns.storage(p, "r") as s:
        np.testing.assert_array_equal(s.read(3), a[:3])
        w = s.read(12)  # wraps past the end
        np.testing.assert_array_equal(w, np.vstack([a, b, a])[3:15])
    with ns.storage(p, "r") as s:
        assert len(s.read(100, wrap=False)) == 12
    # an empty file
    ns.save(tmp_path / "e.mcv", np.zeros((0, 10)))
    assert ns.load(tmp_path / "e.mcv").shape == (0, 10)


def test_bad_files_are_refused(tmp_path):
    p = tmp_path / "x.mcv"
    p.write_bytes(b"not a neutron file" + bytes(2000))
    with pytest.raises(ValueError, match="not a neutron storage"):
        ns.load(p)
    good = open(os.path.join(GOLDEN, "singletestneutron.mcv"), "rb").read()
    p.write_bytes(good[:-8])  # header says 1 neutron, 72 bytes follow
    with pytest.raises(ValueError, match="header says 1"):
        ns.load(p)
    with pytest.raises(ValueError):
        ns.save(tmp_path / "y.mcv", np.zeros(11))


def test_neutron_from_storage_reads_mcv():
    from acc_gb300.components.sources.neutronfromstorage import \
        NeutronFromStorage
    src = NeutronFromStorage(
        "src", os.path.join(GOLDEN, "singletestneutron.mcv"))
    np.testing.assert_array_equal(src.propagate_params[0],
                                  np.arange(10.0)[None])


def test_decode_sorts_and_counts_overflow():
    rows = np.zeros((3, 11))
    rows.view(np.uint64)[:, 0] = [9, 2, 2]
    rows[:, 1:] = [[1.0] * 10, [5.0] * 10, [4.0] * 10]
    buf = np.concatenate([np.zeros(1), rows.reshape(-1)])
    buf[:1].view(np.uint64)[0] = 7  # 7 reached, 3 held
    idx, n, reached = decode(buf)
    assert list(idx) == [2, 2, 9] and reached == 7
    assert list(n[:, 0]) == [4.0, 5.0, 1.0]


def _oracle_saved(ins, ncount, seed=5):
    from oracle import binding as O
    b = HostBinder()
    ch = chain_for_instrument(ins, b)
    st = [c for c in ins.components if isinstance(c, NeutronToStorage)][0]
    _, out, last = O.run_chain(ch, ncount, seed=seed, record=True)
    return decode(b.buffers[(id(st), "rows")]), out, last, ch


def test_oracle_saves_the_neutrons_that_reach_it():
    """Storage as the last component: what it saved is what the chain
    returns for the neutrons that reached it."""
    from acc_gb300.instruments import saved_guide_chain
    ins = saved_guide_chain()
    (idx, saved, reached), out, last, ch = _oracle_saved(ins, 100000)
    reaching = np.nonzero(last == ch.ncomp - 1)[0]
    assert reached == len(saved) == len(reaching) > 1000
    np.testing.assert_array_equal(idx, reaching)
    np.testing.assert_array_equal(saved, out[reaching])


def test_oracle_capacity_overflow_is_counted():
    from oracle import binding as O
    from acc_gb300.components.sources.source_simple import Source_simple
    st = NeutronToStorage("st", capacity=5)
    comps = [Source_simple("s", radius=0.05, dist=1.0, xw=0.05, yh=0.05,
                           E0=52.5, dE=47.5), st]
    b = HostBinder()
    ch = build_chain(comps, binder=b)
    O.run_chain(ch, 100, seed=1)
    idx, saved, reached = decode(b.buffers[(id(st), "rows")])
    assert reached == 100 and len(saved) == 5


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("floattype", ["float64", "float32"])
def test_gpu_saved_neutrons_match_the_oracle(floattype):
    from acc_gb300 import engine
    from acc_gb300.instruments import saved_guide_chain
    n = 500000
    (oidx, osaved, oreached), _, _, _ = _oracle_saved(saved_guide_chain(), n)
    ins = saved_guide_chain()
    st = ins.components[-1]
    st.expect_neutrons(n)
    engine.run_instrument(ins, n, seed=5, floattype=floattype)
    idx, saved, reached = st.stored()
    assert reached == len(saved)
    from helpers import rel_err
    if floattype == "float64":
        # relative to each field's RMS where a value is smaller (a z left
        # by cancellation against 16 m of flight), as the chain tests do
        np.testing.assert_array_equal(idx, oidx)
        assert rel_err(saved, osaved).max() < 1e-12
        return
    # FP32: the same neutrons to a few in 1e4 (float rounding decides a
    # few wall hits), their values within the chain-level bounds of the
    # same-stream parity tests (1e-4 relative, a 1e-3 share excepted)
    common, ia, ib = np.intersect1d(idx, oidx, return_indices=True)
    assert len(common) >= 0.999 * max(len(idx), len(oidx))
    err = rel_err(saved[ia], osaved[ib]).max(axis=1)
    assert (err > 1e-4).sum() <= 1e-3 * len(common), np.sort(err)[-5:]
    assert np.median(err) < 1e-5


@pytest.mark.gpu
def test_gpu_save_then_replay_reproduces_the_monitors(tmp_path):
    """run_script saves the guide-exit neutrons to a .mcv file; replaying
    that file onto the same monitors gives the same histograms."""
    from acc_gb300 import engine, run_script
    n = 1000000
    script = tmp_path / "saved.py"
    script.write_text(
        "from acc_gb300.instruments import saved_guide_chain\n"
        "instrument = saved_guide_chain()\n")
    ins = run_script.run(str(script), str(tmp_path / "out"), n, _acc_seed=3)
    path = tmp_path / "out" / "after_guide2.mcv"
    saved = ns.load(path)
    st = ins.components[-1]
    assert len(saved) == st.stored()[2] > 10000
    from acc_gb300.instruments import guide_exit_replay
    rep = guide_exit_replay(str(path))
    engine.run_instrument(rep, len(saved), seed=1)
    for a, b in ((ins.components[3], rep.components[1]),
                 (ins.components[4], rep.components[2])):
        np.testing.assert_array_equal(a.out[0], b.out[0])
        np.testing.assert_allclose(a.out[1:], b.out[1:], rtol=1e-12,
                                   atol=0)


def _ms_saved(capacity):
    """The multiple-scattering test instrument with its outputs saved at
    the 4pi monitor's position: several rows share an incident neutron's
    index."""
    from acc_gb300.instruments import ms_hollow_cylinder
    ins = ms_hollow_cylinder()
    ins.append(NeutronToStorage("after_sample", capacity=capacity),
               position=(0, 0, 2.0))
    return ins


def test_oracle_saves_every_output_of_a_multiple_scatterer():
    (idx, saved, reached), _, _, _ = _oracle_saved(_ms_saved(200000), 5000)
    assert reached == len(saved) > 5000
    counts = np.bincount(idx.astype(np.int64))
    assert counts.max() > 1  # fan-out: rows share an index
    assert np.all(np.diff(idx.astype(np.int64)) >= 0)


@pytest.mark.gpu
def test_gpu_multiple_scatterer_outputs_match_the_oracle():
    """FP64: the same rows (index, then values) as the oracle, to 1e-12."""
    from acc_gb300 import engine
    from helpers import rel_err
    n = 20000
    (oidx, osaved, oreached), _, _, _ = _oracle_saved(_ms_saved(500000), n)
    ins = _ms_saved(500000)
    engine.run_instrument(ins, n, seed=5, floattype="float64")
    idx, saved, reached = ins.components[-1].stored()
    assert reached == oreached == len(saved)
    np.testing.assert_array_equal(idx, oidx)
    assert rel_err(saved, osaved).max() < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("floattype", ["float64", "float32"])
def test_gpu_buffered_process_saves_its_input(floattype):
    """ComponentBase.process (the buffered mode) on a NeutronToStorage:
    it passes the neutrons through and saves each under its index."""
    from acc_gb300 import engine
    from acc_gb300.components import ComponentBase as CB
    from acc_gb300.instruments import stored_neutrons
    a = stored_neutrons(n=3001)
    st = NeutronToStorage("st", capacity=4000)
    old = CB.ComponentBase._floattype
    CB.change_floattype(floattype)
    try:
        out = st.process(a)
    finally:
        CB.change_floattype(old)
    idx, saved, reached = st.stored()
    assert reached == len(saved) == len(a)
    np.testing.assert_array_equal(idx, np.arange(len(a)))
    tol = 1e-15 if floattype == "float64" else 1e-6
    np.testing.assert_allclose(saved, a, rtol=tol, atol=tol * 1e-3)
    np.testing.assert_allclose(out, a, rtol=tol, atol=tol * 1e-3)
