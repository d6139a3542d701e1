"""The SNS source's FP32 inverse tables (acc_gb300/components/sources/
SNS_source.py, fp32_tables) against the oracle's FP64 sampler, which
inverts the cumulative tables per draw with the reference's zero_find
(SNS_source.py:22-106).  The device lookup (sns_generate_f32) is restated
here in NumPy.

Bounds: E from the table within 2e-4 relative of zero_find's E at the same
u (linear interpolation between 4097 nodes of a smooth inverse); t, drawn
by the two-row mixture, follows the oracle's distribution at fixed E
(Kolmogorov-Smirnov distance below 0.02 over 20000 draws each, about 2.8
standard errors); the regular range is the whole unit interval for a
window inside the table and starts above the draws whose bracket leaves
the table (VERDI's 0.1-1000 meV), whose energies the host tabulates per
FP32 draw."""

import os
import warnings

import numpy as np
import pytest

from acc_gb300 import _native as nat
from acc_gb300 import instruments
from acc_gb300.components.sources.SNS_source import SNS_source
from acc_gb300.engine import build_chain
from acc_gb300.memory import HostBinder


@pytest.fixture(scope="module")
def moderator():
    """VERDI's moderator file (the reference's SNS moderator)."""
    return instruments.shipped_moderator(instruments.SNS_MODERATOR)


@pytest.fixture(scope="module")
def short_moderator():
    """A synthetic moderator table that ends at 10 eV, where VERDI's
    0.1-1000 meV window makes the reference's bracket leave the table."""
    path = instruments.synthetic_moderator_file(nE=141, nt=160)
    yield path
    os.remove(path)


def _source(path, Emin, Emax):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        src = SNS_source("m", path, Emin, Emax, 0.03, 0.03, 6.2, 0.1, 0.1)
    comp = build_chain([src], binder=HostBinder()).comp[0]
    ftab, u_lo, u_hi, _, _ = src._fp32
    return src, comp, ftab.astype(np.float64), u_lo, u_hi


def _lookup(ftab, nE, randE, randt, tails=None):
    """sns_generate_f32 (csrc/components.cuh) in float64; `tails` =
    (u_lo, u_hi, n_lo, n_hi) routes draws outside [u_lo, u_hi] (randE a
    multiple of 2^-24 there) to the per-draw tail energies."""
    NE, NT = nat.MCV_SNS_E_NODES, nat.MCV_SNS_T_NODES
    Einv = ftab[:NE + 1]
    Es = ftab[NE + 1:NE + 1 + nE]
    mass = ftab[NE + 1 + nE:NE + 1 + 2 * nE]
    Tinv = ftab[NE + 1 + 2 * nE:NE + 1 + 2 * nE + nE * (NT + 1)].reshape(
        nE, NT + 1)
    tail = ftab[NE + 1 + 2 * nE + nE * (NT + 1):]
    if tails is not None and not tails[0] <= randE <= tails[1]:
        k = int(randE * 2 ** 24)
        n_lo, n_hi = tails[2], tails[3]
        E = tail[k] if k < n_lo else tail[n_lo + k - (2 ** 24 - n_hi)]
    else:
        s = randE * NE
        k = min(int(s), NE - 1)
        E = Einv[k] + (s - k) * (Einv[k + 1] - Einv[k])
    lo = int(np.searchsorted(Es, E, side="left"))
    if lo >= nE:
        El = Eh = nE - 1
        wl = 0.0
    else:
        Eh, El = lo, (lo - 1 if lo > 0 else nE - 1)
        wl = (Es[Eh] - E) / (Es[Eh] - Es[El])
    ml, mh = wl * mass[El], (1 - wl) * mass[Eh]
    pl = ml / (ml + mh)
    row, ut = (El, randt / pl) if randt < pl else (Eh, (randt - pl) / (1 - pl))
    st = min(ut, 1.0) * NT
    j = min(int(st), NT - 1)
    t = Tinv[row, j] + (st - j) * (Tinv[row, j + 1] - Tinv[row, j])
    return E * 1000.0, t * 1e-6


def test_energy_table_follows_zero_find(oracle_lib, moderator):
    from oracle import binding as O
    src, comp, ftab, u_lo, u_hi = _source(moderator, 5.0, 20.0)
    assert (u_lo, u_hi) == (0.0, 1.0)
    for u in np.linspace(0.0, 1.0, 997)[1:-1]:
        E_tab, _ = _lookup(ftab, comp.ip[1], u, 0.5)
        E_ref, _ = O.sns_generate(comp, u, 0.5)
        assert abs(E_tab - E_ref) <= 2e-4 * E_ref, (u, E_tab, E_ref)


def test_verdi_window_on_the_reference_file(oracle_lib, moderator):
    """VERDI's 0.1-1000 meV window lies inside the reference's table
    (1e-5 - 94 eV), so zero_find's bracket never leaves it; the inverse
    spectrum bends sharply near 0.1 meV, and the first intervals, whose
    linear interpolation misses zero_find's midpoint energy by more than
    2e-5, take per-draw tail energies.  Every 24-bit draw then lands within
    2e-4 of zero_find (checked on 2000 draws and on each tail draw's
    neighbourhood of the boundary)."""
    from oracle import binding as O
    src, comp, ftab, u_lo, u_hi = _source(moderator, 0.1, 1000.0)
    _, _, _, n_lo, n_hi = src._fp32
    assert 0.0 < u_lo <= 16 / 4096 and u_hi == 1.0
    assert n_lo == u_lo * 2 ** 24 and n_hi == 0
    tails = (u_lo, u_hi, n_lo, n_hi)
    ks = np.concatenate([np.linspace(1, 2 ** 24 - 1, 2000).astype(int),
                         n_lo + np.arange(-20, 20)])
    for k in ks:
        u = k / 2 ** 24
        E_tab, _ = _lookup(ftab, comp.ip[1], u, 0.5, tails)
        E_ref, _ = O.sns_generate(comp, u, 0.5)
        assert abs(E_tab - E_ref) <= 2e-4 * E_ref, (k, E_tab, E_ref)


def test_regular_range_excludes_the_wandering_draws(oracle_lib,
                                                    short_moderator):
    """VERDI's window on a table that ends at 10 eV: below u_lo the
    reference's bracket expands past the table (energies far above it,
    test_oracle_kats.py); the FP32 kernels look those draws up by k (tail
    table), as they do the top intervals, where the inverse spectrum
    bends too sharply for linear interpolation.  In between the table
    holds."""
    from oracle import binding as O
    src, comp, ftab, u_lo, u_hi = _source(short_moderator, 0.1, 1000.0)
    assert 0.0 < u_lo < 0.01 and 0.99 < u_hi <= 1.0
    below = [O.sns_generate(comp, u, 0.5)[0] for u in
             np.linspace(0.0, u_lo, 50, endpoint=False)]
    assert max(below) > 1e4  # meV: past the table
    for u in np.linspace(u_lo, u_hi, 500)[1:-1]:
        E_tab, _ = _lookup(ftab, comp.ip[1], u, 0.5)
        E_ref, _ = O.sns_generate(comp, u, 0.5)
        assert abs(E_tab - E_ref) <= 2e-4 * E_ref, (u, E_tab, E_ref)


def test_tail_energies_are_zero_finds_at_each_draw(oracle_lib,
                                                   short_moderator):
    """Below u_lo and above u_hi every FP32 draw u = k 2^-24 has its own
    tail entry, zero_find's energy at that u (float32-rounded)."""
    from oracle import binding as O
    src, comp, ftab, u_lo, u_hi = _source(short_moderator, 0.1, 1000.0)
    _, _, _, n_lo, n_hi = src._fp32
    first_hi = int(np.floor(u_hi * 2 ** 24)) + 1
    assert n_lo == int(np.ceil(u_lo * 2 ** 24)) > 0
    assert n_hi == 2 ** 24 - first_hi > 0
    assert n_lo + n_hi <= nat.MCV_SNS_TAIL_MAX
    assert (comp.dp[18], comp.dp[19]) == (n_lo, n_hi)
    nE, NE, NT = comp.ip[1], nat.MCV_SNS_E_NODES, nat.MCV_SNS_T_NODES
    tail = ftab[NE + 1 + 2 * nE + nE * (NT + 1):]
    assert len(tail) == n_lo + n_hi
    for k in list(range(0, n_lo, 997)) + [n_lo - 1]:
        E_ref, _ = O.sns_generate(comp, k / 2 ** 24, 0.5)
        assert abs(tail[k] * 1000.0 - E_ref) <= 1e-6 * E_ref, (k, E_ref)
    for k in list(range(first_hi, 2 ** 24, 997)) + [2 ** 24 - 1]:
        E_ref, _ = O.sns_generate(comp, k / 2 ** 24, 0.5)
        e = tail[n_lo + k - first_hi] * 1000.0
        assert abs(e - E_ref) <= 1e-6 * E_ref, (k, E_ref)
    # a window inside the table needs no tail
    src2, comp2, _, _, _ = _source(short_moderator, 5.0, 20.0)
    assert src2._fp32[3:] == (0, 0) and comp2.dp[18] == comp2.dp[19] == 0


@pytest.mark.parametrize("randE", [0.05, 0.3, 0.62, 0.97])
def test_time_mixture_matches_the_reference_distribution(oracle_lib,
                                                         moderator, randE):
    from oracle import binding as O
    src, comp, ftab, u_lo, u_hi = _source(moderator, 0.1, 1000.0)
    rng = np.random.default_rng(7)
    n = 20000
    ut = rng.random(n)
    t_tab = np.array([_lookup(ftab, comp.ip[1], randE, x)[1] for x in ut])
    t_ref = np.array([O.sns_generate(comp, randE, x)[1]
                      for x in rng.random(n)])
    a, b = np.sort(t_tab), np.sort(t_ref)
    grid = np.concatenate([a, b])
    ks = np.max(np.abs(np.searchsorted(a, grid, side="right") / n
                       - np.searchsorted(b, grid, side="right") / n))
    assert ks < 0.02, ks


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["short", "reference"])
def test_gpu_tail_draws_take_their_tail_energy(engine_lib, which,
                                               short_moderator, moderator):
    """The FP32 kernel's tail lookup (sns_generate_f32: the k < n_lo
    branch and the n_lo + k - (2^24 - n_hi) branch), through injected
    uniforms: a neutron whose energy uniform is k 2^-24 outside [u_lo,
    u_hi] leaves the source with tail[k]'s energy (within float rounding of
    v = SE2V sqrt(E))."""
    import acc_gb300
    from acc_gb300 import engine
    from acc_gb300.conversion import VS2E
    path = short_moderator if which == "short" else moderator
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        src = SNS_source("m", path, 0.1, 1000., 0.03, 0.03, 6.2, 0.1, 0.1)
    ins = acc_gb300.instrument()
    ins.append(src)
    chain = engine.chain_for_instrument(ins)  # packs the FP32 tables
    ftab, u_lo, u_hi, n_lo, n_hi = src._fp32
    nE, NE, NT = len(src.propagate_params[9]), nat.MCV_SNS_E_NODES, \
        nat.MCV_SNS_T_NODES
    tail = ftab[NE + 1 + 2 * nE + nE * (NT + 1):].astype(np.float64)
    first_hi = 2 ** 24 - n_hi
    ks = [0, 1, n_lo // 2, n_lo - 1]
    if n_hi:
        ks += [first_hi, first_hi + n_hi // 2, 2 ** 24 - 1]
    expect = [tail[k] if k < n_lo else tail[n_lo + k - first_hi] for k in ks]
    u = np.full((len(ks), 6), 0.5, np.float32)
    u[:, 4] = np.array(ks, np.float64) / 2 ** 24
    out, _ = engine.replay(chain, len(ks), uniforms=u, floattype="float32")
    out = out.cpu().numpy()
    E = VS2E * (out[:, 3:6] ** 2).sum(axis=1)
    np.testing.assert_allclose(E, np.array(expect) * 1000.0, rtol=1e-6)
