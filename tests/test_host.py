"""Host-side logic: instrument geometry, component packing, the mcvine
alias and run_script's script loading (no GPU)."""

import json
import os
import textwrap

import numpy as np
import pytest

import acc_gb300
from acc_gb300 import _native as nat
from acc_gb300.components.monitors.psd_monitor import PSD_monitor
from acc_gb300.components.optics.arm import Arm
from acc_gb300.components.optics.guide import Guide
from acc_gb300.components.sources.source_simple import Source_simple
from acc_gb300.engine import build_chain
from acc_gb300.instrument import applyTransformation, calcTransformations
from acc_gb300.memory import HostBinder

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))


def test_coordinate_transforms_match_reference_kats():
    g = KATS["coord_transform"]
    ins = acc_gb300.instrument()
    comps = []
    for i, pl in enumerate(g["placements"]):
        a = Arm(f"comp{i + 1}")
        rel = comps[pl["relative"]] if pl["relative"] is not None else None
        ins.append(a, position=pl["position"], orientation=pl["orientation"],
                   relativeTo=rel)
        comps.append(a)
    offsets, rotmats = calcTransformations(ins)
    assert len(offsets) == len(rotmats) == len(comps) - 1
    for hop in g["hops"]:
        r = np.array(hop["r"], float)
        v = np.array(hop["v"], float)
        k = hop["hop"]
        applyTransformation(r, v, rotmats[k], offsets[k])
        np.testing.assert_allclose(r, hop["r1"], atol=1e-12)
        np.testing.assert_allclose(v, hop["v1"], atol=1e-12)


def test_source_simple_params_and_checks():
    s = Source_simple("s", radius=0.05, dist=5, xw=0.01, yh=0.01, E0=60, dE=10)
    (square, width, height, radius, wl, L0, dL, E0, dE, xw, yh, dist,
     pmul) = s.propagate_params
    assert not square and not wl
    assert pmul == pytest.approx(1e4 * np.pi * 0.05 ** 2)
    with pytest.raises(RuntimeError):
        Source_simple("s", radius=0.05, width=0.1, height=0.1)
    with pytest.raises(RuntimeError):
        Source_simple("s", radius=0.05, E0=10, dE=20)
    with pytest.raises(RuntimeError):
        Source_simple("s", radius=0.05, E0=0, dE=0, Lambda0=1, dLambda=2)
    sq = Source_simple("s", radius=0, width=0.01, height=0.02, E0=60, dE=1)
    assert sq.propagate_params[0] is True


def test_guide_params():
    g = Guide("g", w1=0.05, h1=0.05, w2=0.02, h2=0.02, l=5, m=3, alpha=3)
    assert g.propagate_params == pytest.approx(
        (-0.015, -0.015, 0.025, 0.025, 5, 0.99, 0.0219, 3, 3, 0.003))


def test_build_chain_packs_transforms_and_tallies():
    ins = acc_gb300.instrument()
    src = Source_simple("s", radius=0.05, dist=1, xw=0.05, yh=0.05, E0=52.5,
                        dE=47.5)
    g = Guide("g", 0.05, 0.05, 0.05, 0.05, 10, m=3, alpha=3)
    mon = PSD_monitor("m", xwidth=0.06, yheight=0.06, nx=100, ny=100)
    ins.append(src, position=(0, 0, 0))
    ins.append(g, position=(0, 0, 1))
    ins.append(mon, position=(0, 0, 11.001), orientation=(0, 0, 90))
    b = HostBinder()
    off, rot = calcTransformations(ins)
    ch = build_chain(ins.components, off, rot, b)
    assert ch.ncomp == 3
    assert ch.comp[1].flags & nat.FLAG_IDENTITY_ROT
    assert not ch.comp[2].flags & nat.FLAG_IDENTITY_ROT
    assert ch.off[1][2] == 1.0 and ch.off[2][2] == pytest.approx(10.001)
    assert ch.comp[2].ip[0] == 100 and ch.comp[2].ip[1] == 100
    assert ch.comp[2].tally == b.tallies[id(mon)].ctypes.data
    assert b.out(mon).shape == (3, 100, 100)
    for k in range(11):
        assert ch.comp[0].fp[k] == pytest.approx(ch.comp[0].dp[k], rel=1e-7)


def test_build_chain_limits():
    with pytest.raises(ValueError):
        build_chain([], binder=HostBinder())
    with pytest.raises(ValueError):
        build_chain([Arm(f"a{i}") for i in range(nat.MCV_MAX_COMPONENTS + 1)],
                    binder=HostBinder())


def test_mcvine_alias_and_script_loading(tmp_path):
    from acc_gb300 import compat
    from acc_gb300.run_script import loadInstrument
    script = tmp_path / "instr.py"
    script.write_text(textwrap.dedent('''
        import mcvine
        from mcvine.acc.components.sources.source_simple import Source_simple
        from mcvine.acc.components.optics.guide import Guide
        from mcvine.acc.components.monitors.psd_monitor import PSD_monitor

        def instrument(z_mon=12., guide_m=3):
            ins = mcvine.instrument()
            ins.append(Source_simple('src', radius=0., width=0.03, height=0.03,
                       dist=1., xw=0.035, yh=0.035, Lambda0=10., dLambda=9.5,
                       E0=0., dE=0.), position=(0, 0, 0))
            ins.append(Guide('g', w1=0.035, h1=0.035, w2=0.035, h2=0.035,
                             l=10, m=guide_m), position=(0, 0, 1.))
            ins.append(PSD_monitor('m', xwidth=0.08, yheight=0.08),
                       position=(0, 0, z_mon))
            return ins
    '''))
    assert compat.install_mcvine_alias() in (True, False)
    with pytest.warns(UserWarning):
        ins = loadInstrument(str(script), z_mon=13., unknown_kw=1)
    names = [type(c).__name__ for c in ins.components]
    assert names == ["Source_simple", "Guide", "PSD_monitor"]
    off, rot = calcTransformations(ins)
    np.testing.assert_allclose(off[1], [0, 0, 12.])


def test_monitor_axes():
    m = PSD_monitor("m", xmin=-0.03, xmax=0.03, ymin=-0.03, ymax=0.03, nx=100,
                    ny=50)
    assert m.x_centers.size == 100 and m.y_centers.size == 50
    assert m.x_centers[0] == pytest.approx(-0.03 + 0.0003)
    h = m.getHistogram(1.0)
    assert h.data.shape == (100, 50)


def test_sharding_ranges_cover_exactly():
    from acc_gb300.sharding import shard_range
    for n, w in [(10, 3), (1, 4), (1_000_003, 8), (0, 2)]:
        parts = [shard_range(n, r, w) for r in range(w)]
        assert sum(c for _, c in parts) == n
        pos = 0
        for f, c in parts:
            assert f == pos
            pos += c


def test_chi2_and_z_scores_of_independent_tallies():
    from acc_gb300.stats import chi2_per_dof, z_summary
    rng = np.random.default_rng(0)

    def tally(n):
        # 400 bins, Poisson entries with exponential weights
        cnt = rng.poisson(200, 400).astype(float)
        w = [rng.exponential(1.0, int(c)) for c in cnt]
        return np.stack([cnt, [x.sum() for x in w],
                         [(x * x).sum() for x in w]])

    a, b = tally(0), tally(0)
    c2, dof = chi2_per_dof(a, b)
    z = z_summary(a, b)
    assert dof == 400 and abs(c2 - 1) < 0.25
    assert abs(z["mean_z"]) < 0.2 and abs(z["std_z"] - 1) < 0.15
    assert z["frac_abs_z_gt_3"] < 0.02
    b2 = b.copy()
    b2[1] *= 1.5  # a 50% bias is seen
    assert chi2_per_dof(a, b2)[0] > 3


def test_weight_exp2_places_the_source_weight_near_2_64():
    from acc_gb300 import engine, instruments
    for name in ("guide_chain", "sphere_theta_tof", "sqe_hollow_cylinder"):
        comps = getattr(instruments, name)().components
        e = engine.weight_exp2(comps)
        w = comps[0].nominal_weight()
        assert abs(np.log2(w) + e - engine.WEIGHT_TARGET_EXP2) <= 0.5
        ch = build_chain(comps, binder=HostBinder())
        assert ch.weight_exp2 == e
    # no source first: no scaling
    assert engine.weight_exp2([Arm("a")]) == 0


def test_leading_arms_are_left_out_of_the_chain():
    """An arm ahead of the source (as VERDI's origin) is not in the chain;
    the transforms of the kept components are unchanged."""
    from acc_gb300 import instruments as I
    from acc_gb300.engine import chain_for_instrument, chain_parts
    from acc_gb300.instrument import calcTransformations
    ins = I.verdi(moderator_file=I.synthetic_moderator_file(nE=20, nt=20))
    comps, off, rot, first = chain_parts(ins)
    assert first == 1 and comps[0] is ins.components[1]
    off_all, rot_all = calcTransformations(ins)
    np.testing.assert_array_equal(off, off_all[1:])
    np.testing.assert_array_equal(rot, rot_all[1:])
    ch = chain_for_instrument(ins, HostBinder())
    assert ch.ncomp == len(ins.components) - 1 == 25
    assert ch.first_component == 1
    assert ch.comp[0].opcode == nat.OP_SNS_SOURCE
    # the FP32 weight scale comes from the source's nominal weight
    assert ch.weight_exp2 != 0


def test_verdi_mirror_geometry():
    """The elliptic profile (acc/test/ellipse.py:101-162) is continuous from
    segment to segment and the shield tip lies on both sight lines of
    SingleWall.calc_shield_xz (:37-54)."""
    from acc_gb300 import instruments as I
    a, b = 0.105, 15.875
    h1, h2, w1, w2 = I.elliptic_guide_segments(b, 6.35, 16.0, 500, 2 * b, 2 * a)
    np.testing.assert_allclose(h2[:-1], h1[1:], rtol=1e-12)
    np.testing.assert_array_equal(h1, w1)
    np.testing.assert_allclose(h1[0], 2 * a * np.sqrt(6.35 / b * (2 - 6.35 / b)))
    x, z = I.shield_vertex(a, b, 0., 0.03, 6.35, 26.9, 31.75, 0.02)
    xe = I.ellipse_half_opening(26.9, a, b)
    xs = I.ellipse_half_opening(6.35, a, b)
    # on the line (0, -0.015) -> (26.9, xe) and on (6.35, xs) -> (31.75, -0.01)
    np.testing.assert_allclose(x, -0.015 + (xe + 0.015) * z / 26.9, rtol=1e-12)
    np.testing.assert_allclose(
        x, xs + (-0.01 - xs) * (z - 6.35) / (31.75 - 6.35), rtol=1e-12)
    assert 6.35 < z < 26.9


def test_chain_keeps_its_tables_alive():
    """A chain built from a temporary instrument holds the components whose
    lookup tables its pointers refer to."""
    import gc
    import weakref
    from acc_gb300 import instruments as I
    from acc_gb300.engine import chain_for_instrument
    ch = chain_for_instrument(I.tapered_guide_chain(), HostBinder())
    guide = weakref.ref(ch._components[1])
    gc.collect()
    assert guide() is not None
    assert ch.comp[1].table != 0


def test_tapered_guide_quiet_blocks():
    """A guide of QUIET_MIN_SEGMENTS segments or more packs ip[1] = 16 and,
    after the 10 x nseg rows, each block's narrowest width and height; a
    shorter one packs neither.  The engine rejects a table missing the
    block rows."""
    import ctypes
    from acc_gb300.components.optics.guide_tapering import Guide
    n = 300
    z = np.linspace(0.0, 1.0, n)
    w1 = 0.03 + 0.01 * np.sin(3 * z)
    w2 = np.roll(w1, -1)
    h1 = 0.04 - 0.01 * z
    h2 = h1 - 0.0001
    g = Guide("g", l=10.0, segments=(h1, h2, w1, w2))
    ch = build_chain([g], binder=HostBinder())
    c = ch.comp[0]
    assert (c.ip[0], c.ip[1]) == (n, 16)
    nblk = -(-n // 16)
    assert c.table_len == 10 * n + 2 * nblk
    flat = np.ctypeslib.as_array(ctypes.cast(c.table, ctypes.POINTER(
        ctypes.c_double)), shape=(c.table_len,))
    rows = flat[10 * n:].reshape(2, nblk)
    for b in range(nblk):
        s = slice(16 * b, min(16 * b + 16, n))
        assert rows[0, b] == min(w1[s].min(), w2[s].min())
        assert rows[1, b] == min(h1[s].min(), h2[s].min())
    short = Guide("s", l=1.0, segments=(h1[:100], h2[:100], w1[:100],
                                         w2[:100]))
    c2 = build_chain([short], binder=HostBinder()).comp[0]
    assert c2.ip[1] == 0 and c2.table_len == 1000
    # mcv_run_chain validates the chain before it looks at the context
    import ctypes as C
    L = nat.lib()
    st = nat.mcv_status()
    c.table_len = 10 * n
    rc = L.mcv_run_chain(None, C.byref(ch), 1, 0, 0, 32, None, None,
                         C.byref(st))
    with pytest.raises(nat.EngineError, match="block rows"):
        nat.check(rc, st)
    c.table_len = 10 * n + 2 * nblk
    rc = L.mcv_run_chain(None, C.byref(ch), 1, 0, 0, 32, None, None,
                         C.byref(st))
    with pytest.raises(nat.EngineError, match="context is NULL"):
        nat.check(rc, st)


def test_isotropic_box():
    """IsotropicBox (isotropic_box.py) is the single scatterer on a box with
    the isotropic kernel."""
    from acc_gb300.components.samples.isotropic_box import IsotropicBox
    ch = build_chain([IsotropicBox("b", 0.02, 0.03, 0.004, 10.0, 20.0)],
                     binder=HostBinder())
    c = ch.comp[0]
    assert c.opcode == nat.OP_HSS and c.ip[1] == nat.KERNEL_ISOTROPIC
    assert c.ip[2] == nat.SHAPE_BOX
    assert [c.dp[k] for k in (0, 1, 2, 8, 9)] == [0.02, 0.03, 0.004, 10.0, 20.0]


# every component module of the reference's acc/components that an
# instrument script imports, with the name it takes from it (the earlier
# guide implementations guide_baseline, numpy_guide and oo_guide, superseded
# by guide.py in the reference, are not provided)
REFERENCE_COMPONENTS = [
    ("monitors.iqe_monitor", "IQE_monitor"),
    ("monitors.posdiv_monitor", "PosDiv_monitor"),
    ("monitors.psd_monitor", "PSD_monitor"),
    ("monitors.psd_monitor_4pi", "PSD_monitor_4Pi"),
    ("monitors.wavelength_monitor", "Wavelength_monitor"),
    ("optics.arm", "Arm"),
    ("optics.beamstop", "Beamstop"),
    ("optics.guide", "Guide"),
    ("optics.guide_anyshape", "Guide_anyshape"),
    ("optics.guide_anyshape_gravity", "Guide_anyshape_gravity"),
    ("optics.guide_tapering", "Guide"),
    ("optics.slit", "Slit"),
    ("samples.homogeneous_multiple_scatterer", "factory"),
    ("samples.homogeneous_single_scatterer", "factory"),
    ("samples.isotropic_box", "IsotropicBox"),
    ("sources.SNS_source", "SNS_source"),
    ("sources.STS_source", "STS_source"),
    ("sources.neutronfromstorage", "NeutronFromStorage"),
    ("sources.source_simple", "Source_simple"),
]


@pytest.mark.parametrize("module,name", REFERENCE_COMPONENTS)
def test_reference_component_paths_import(module, name):
    import importlib
    from acc_gb300 import compat
    compat.install_mcvine_alias(force=True)
    m = importlib.import_module("mcvine.acc.components." + module)
    assert callable(getattr(m, name))
    assert getattr(m, "category", module.split(".")[0]) == \
        module.split(".")[0]


def test_run_keywords_reach_the_instrument(tmp_path):
    """run_script.run passes every keyword to the instrument factory (the
    reference's run_script.py:10-35, 297-328): `seed` and `floattype` are
    instrument keywords like any other; the engine's own overrides are
    `_acc_seed` / `_acc_floattype`."""
    import inspect
    from acc_gb300 import run_script
    params = inspect.signature(run_script.run).parameters
    assert "seed" not in params and "floattype" not in params
    script = tmp_path / "ins.py"
    script.write_text(
        "import acc_gb300\n"
        "from acc_gb300.components.optics.arm import Arm\n"
        "def instrument(seed=0, floattype='x'):\n"
        "    ins = acc_gb300.instrument()\n"
        "    ins.append(Arm('a'))\n"
        "    ins.got = (seed, floattype)\n"
        "    return ins\n")
    ins = run_script.loadInstrument(str(script), seed=5, floattype="y")
    assert ins.got == (5, "y")


def test_additional_kargs_file(tmp_path):
    """--additional-kargs reads a YAML file (JSON when PyYAML is absent)."""
    from acc_gb300 import run_script
    f = tmp_path / "k.yml"
    f.write_text('{"Ei": 60.0, "seed": 3}')
    assert run_script.load_additional_kargs(str(f)) == {"Ei": 60.0, "seed": 3}
    (tmp_path / "e.yml").write_text("")
    assert run_script.load_additional_kargs(str(tmp_path / "e.yml")) == {}
