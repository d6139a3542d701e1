"""The mesh guide (acc/components/optics/guide_anyshape.py) on the oracle:
the reference's tests restated (tests/components/optics/
test_guide_anyshape.py), with the meshes of their data files generated
here (the same vertices and faces)."""

import numpy as np
import pytest

from acc_gb300.components.optics.guide_anyshape import (
    Guide_anyshape, box_guide_mesh, get_faces_data,
    load_scaled_centered_faces, write_off)
from acc_gb300.engine import build_chain
from acc_gb300.memory import HostBinder


@pytest.fixture
def example1(tmp_path):
    """guide_anyshape_example1.off: a 2 x 2 cm channel from z = 1 to 2."""
    path = str(tmp_path / "example1.off")
    write_off(path, *box_guide_mesh(0.02, 0.02, 0.02, 0.02, 1.0, z0=1.0))
    return path


def test_load_scaled_centered_faces(example1):
    """test_guide_anyshape.py:12-61."""
    original = np.array([
        [[-0.01, -0.01, 1.], [-0.01, 0.01, 1.], [-0.01, 0.01, 2.],
         [-0.01, -0.01, 2.]],
        [[-0.01, 0.01, 1.], [0.01, 0.01, 1.], [0.01, 0.01, 2.],
         [-0.01, 0.01, 2.]],
        [[0.01, -0.01, 1.], [0.01, -0.01, 2.], [0.01, 0.01, 2.],
         [0.01, 0.01, 1.]],
        [[-0.01, -0.01, 1.], [-0.01, -0.01, 2.], [0.01, -0.01, 2.],
         [0.01, -0.01, 1.]]])
    c = np.array([0, 0, 1.5])
    f = load_scaled_centered_faces
    assert np.allclose(f(example1), original)
    assert np.allclose(f(example1, xwidth=0.04), (original - c) * 2 + c)
    assert np.allclose(f(example1, zdepth=3), (original - c) * 3 + c)
    with pytest.raises(ValueError):
        f(example1, xwidth=0.04, zdepth=3)
    want = original - c
    want[:, :, 0] *= 2
    want[:, :, 1] *= 3
    want[:, :, 2] *= 4
    assert np.allclose(f(example1, 0.04, 0.06, 4), want + c)
    assert np.allclose(f(example1, center=True), original - c)
    assert np.allclose(f(example1, xwidth=0.04, center=True),
                       (original - c) * 2)
    assert np.allclose(f(example1, 0.04, 0.06, 4, center=True), want)


def _comp(path):
    return build_chain([Guide_anyshape("g", geometry=path)],
                       binder=HostBinder()).comp[0]


def test_propagate_one_face(oracle_lib, tmp_path):
    """test_guide_anyshape.py:63-107: one face in the y = 0 plane (its unit
    vectors come out as the test's: z, x and the normal y); a neutron
    0.01 m above it, falling at 1 m/s while moving 2000 m/s along z,
    reflects at t = 0.01 s with R0."""
    from oracle import binding as O
    path = str(tmp_path / "face.off")
    write_off(path, np.array([[-1, 0, -1], [-1, 0, 1], [1, 0, 1],
                              [1, 0, -1]], dtype=float), [[0, 1, 2, 3]])
    _, _, unitvecs, faces2d = get_faces_data(path)
    assert np.allclose(unitvecs[0], [[0, 0, 1], [1, 0, 0], [0, 1, 0]])
    # the same square as the test's hand-written polygon
    assert sorted(map(tuple, faces2d[0].round(12))) == \
        [(-1, -1), (-1, 1), (1, -1), (1, 1)]
    st, over = O.anyshape_one(_comp(path),
                              [0, 0.01, -20, 0, -1, 2000, 0, 0, 0, 1])
    assert over == 0
    assert np.allclose(st, [0, 0, 0, 0, 1, 2000, 0, 0, 0.01, 0.99])


def test_propagate_straight_guide(oracle_lib, tmp_path):
    """test_guide_anyshape.py:109-140: the 3.5 x 3.5 cm x 10 m straight
    mesh; a neutron entering at the top edge with vy = 17.5 m/s bounces at
    z = 0, 2, 4, 6, 8 and misses the last face by a hair (vz 1e-10 above
    1000 m/s), stopping at z = 8 with weight (R above m Qc)^5 < 5e-18."""
    from oracle import binding as O
    path = str(tmp_path / "straight.off")
    write_off(path, *box_guide_mesh(0.035, 0.035, 0.035, 0.035, 10.0))
    st, over = O.anyshape_one(
        _comp(path), [0, 0, -1, 0, 0.035 / 2 * 1000, 1000 + 1e-10, 0, 0, 0,
                      1])
    assert over == 0
    assert np.allclose(st[:-1], [0, 0.0175, 8, 0, -17.5, 1000, 0, 0, 0.009])
    assert 0 < st[-1] < 5e-18


@pytest.mark.parametrize("w2", [0.035, 0.04])
def test_box_mesh_equals_the_plain_guide(oracle_lib, tmp_path, w2):
    """A four-face mesh of a rectangular channel is the plain guide
    (guide.py): on the same Philox stream both give the same state on the
    monitor's plane to 1e-9 (the mesh backs off 1e-14 of each flight).  In
    a tapering channel a neutron reflected into a corner can find the
    neighbouring wall's plane behind it (t <= 0, no candidate) and leave
    through the corner, as the reference's mesh algorithm lets it; those
    stay below 0.5%."""
    from acc_gb300 import instruments
    from acc_gb300.components.monitors.psd_monitor import PSD_monitor
    from acc_gb300.components.optics.guide import Guide
    from acc_gb300.components.sources.source_simple import Source_simple
    from acc_gb300.engine import chain_for_instrument
    from acc_gb300.instrument import instrument
    from oracle import binding as O
    path = str(tmp_path / "box.off")
    write_off(path, *box_guide_mesh(0.035, 0.035, w2, w2, 10.0))
    coat = dict(R0=0.99, Qc=0.0219, alpha=6.07, m=3, W=0.003)
    out = []
    for g in (Guide_anyshape("g", geometry=path, **coat),
              Guide("g", w1=0.035, h1=0.035, w2=w2, h2=w2, l=10.0, **coat)):
        ins = instrument("cmp")
        ins.append(Source_simple("s", radius=0.0, width=0.01, height=0.01,
                                 dist=0.9, xw=0.01, yh=0.01, Lambda0=4.0,
                                 dLambda=3.0), position=(0, 0, 0))
        ins.append(g, position=(0, 0, 1.0))
        ins.append(PSD_monitor("m", nx=10, ny=10, xwidth=0.1, yheight=0.1),
                   position=(0, 0, 12.0))
        ch = chain_for_instrument(ins, HostBinder())
        _, o, last = O.run_chain(ch, 20000, seed=9, record=True)
        out.append((o, last))
    (a, la), (b, lb) = out
    alive = (la == 2) & (lb == 2) & (a[:, 9] > 0) & (b[:, 9] > 0)
    assert alive.sum() > 10000
    np.testing.assert_array_equal(la, lb)

    def at_plane(o):
        # the states on the monitor's plane: a neutron that touches no face
        # stays where the mesh guide found it (the reference leaves it
        # there), the plain guide first moves it to its entrance
        dt = -o[:, 2] / o[:, 5]
        return np.stack([o[:, 0] + o[:, 3] * dt, o[:, 1] + o[:, 4] * dt,
                         o[:, 3], o[:, 4], o[:, 5], o[:, 8] + dt, o[:, 9]], 1)
    pa, pb = at_plane(a[alive]), at_plane(b[alive])
    if w2 == 0.035:
        np.testing.assert_allclose(pa, pb, rtol=1e-9, atol=1e-12)
    else:
        same = np.all(np.isclose(pa, pb, rtol=1e-9, atol=1e-12), axis=1)
        assert (~same).mean() < 5e-3, (~same).sum()


def test_gravity_one_face(oracle_lib, tmp_path):
    """guide_anyshape_gravity.py with g = -9.8 m/s^2 along y: a neutron
    0.01 m above the y = 0 face, falling at 1 m/s and moving 2000 m/s
    along z, reaches it at t = 0.009552841750957684 s (the reference's
    test_intersect, tests/components/optics/test_guide_anyshape_gravity.py
    :12-27), reflects with R0 and is then carried along its parabola to
    the mesh's largest z (1 m) without advancing its time."""
    from acc_gb300.components.optics.guide_anyshape import \
        Guide_anyshape_gravity
    from oracle import binding as O
    path = str(tmp_path / "face.off")
    write_off(path, np.array([[-1, 0, -1], [-1, 0, 1], [1, 0, 1],
                              [1, 0, -1]], dtype=float), [[0, 1, 2, 3]])
    g = Guide_anyshape_gravity("g", geometry=path, gravity=(0, -9.8, 0))
    comp = build_chain([g], binder=HostBinder()).comp[0]
    st, over = O.anyshape_one(comp, [0, 0.01, -20, 0, -1, 2000, 0, 0, 0, 1])
    t_hit = 0.009552841750957684
    assert over == 0
    np.testing.assert_allclose(st[8], t_hit, rtol=1e-12)
    z_hit = -20 + 2000 * t_hit
    vy = 1 + 9.8 * t_hit  # reflected
    dt = (1 - z_hit) / 2000
    np.testing.assert_allclose(
        st, [0, vy * dt - 4.9 * dt * dt, 1, 0, vy - 9.8 * dt, 2000, 0, 0,
             t_hit, 0.99], rtol=1e-9, atol=1e-13)


def test_gravity_falls_back_onto_the_same_face(oracle_lib, tmp_path):
    """Under gravity a neutron can hit the face it has just left: a slow
    neutron bouncing along a long floor makes several reflections off the
    one face, each at the parabola's apex spacing 2 vy / g."""
    from acc_gb300.components.optics.guide_anyshape import \
        Guide_anyshape_gravity
    from oracle import binding as O
    path = str(tmp_path / "floor.off")
    write_off(path, np.array([[-1, 0, 0], [-1, 0, 10], [1, 0, 10],
                              [1, 0, 0]], dtype=float), [[0, 1, 2, 3]])
    g = Guide_anyshape_gravity("g", geometry=path, gravity=(0, -9.8, 0))
    comp = build_chain([g], binder=HostBinder()).comp[0]
    # starts on the floor plane's level going up 0.5 m/s, 10 m/s along z
    st, over = O.anyshape_one(comp, [0, 1e-9, 0.0, 0, 0.5, 10.0, 0, 0, 0, 1])
    period = 2 * 0.5 / 9.8
    nref = int(10 / 10 / period)  # reflections within the 10 m floor
    assert nref == 9
    np.testing.assert_allclose(st[8], nref * period, rtol=1e-6)
    np.testing.assert_allclose(st[9], 0.99 ** nref, rtol=1e-9)
