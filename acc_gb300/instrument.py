"""A minimal instrument and geometer.

Restates what mcvine.instrument() / mcni.Instrument provide to the
reference's run_script (acc/run_script.py:141-162): a list of components,
each with a position and orientation, absolute or relative to an earlier
component, and the offset/rotation pairs that take a neutron from one
component's frame to the next one's (r' = R (r - o), v' = R v;
acc/neutron.py:18-23).

Orientation (rx, ry, rz) in degrees uses the McStas rotation convention
(rotate about x, then y, then z; the matrix maps parent-frame coordinates to
the rotated frame's).  The reference's own test
(tests/test_coord_transform_among_comps.py:25-57) pins the single-axis cases.
"""

import math

import numpy as np


def rotation_matrix(orientation):
    """Parent-frame -> local-frame coordinate matrix for (rx, ry, rz) deg."""
    rx, ry, rz = (math.radians(float(a)) for a in orientation)
    cx, sx = math.cos(rx), math.sin(rx)
    cy, sy = math.cos(ry), math.sin(ry)
    cz, sz = math.cos(rz), math.sin(rz)
    return np.array([
        [cy * cz, sx * sy * cz + cx * sz, sx * sz - cx * sy * cz],
        [-cy * sz, cx * cz - sx * sy * sz, sx * cz + cx * sy * sz],
        [sy, -sx * cy, cx * cy],
    ])


class Geometer:
    def __init__(self):
        self._abs = {}

    def register(self, comp, position, orientation, relative_to):
        M_rel = rotation_matrix(orientation)
        p = np.asarray(position, dtype=float)
        if relative_to is None:
            P, M = p, M_rel
        else:
            Pr, Mr = self._abs[id(relative_to)]
            P = Pr + Mr.T @ p
            M = M_rel @ Mr
        self._abs[id(comp)] = (P, M)

    def position(self, comp):
        return self._abs[id(comp)][0]

    def rotation(self, comp):
        return self._abs[id(comp)][1]

    def orientation(self, comp):
        return self.rotation(comp)


class Instrument:
    """Ordered components with placements (mcni.Instrument stand-in)."""

    def __init__(self, name="instrument"):
        self.name = name
        self.components = []
        self.geometer = Geometer()

    def append(self, component, position=(0, 0, 0), orientation=(0, 0, 0),
               relativeTo=None):
        if relativeTo is not None and not any(
                relativeTo is c for c in self.components):
            raise ValueError("relativeTo must be a component already appended")
        self.components.append(component)
        self.geometer.register(component, position, orientation, relativeTo)
        return component

    def __repr__(self):
        names = ", ".join(getattr(c, "name", "?") for c in self.components)
        return f"Instrument({names})"


def instrument(name="instrument"):
    return Instrument(name)


def relative_transform(geometer, a, b):
    """(offset, rotmat) taking a neutron from a's frame to b's frame."""
    Pa, Ma = geometer.position(a), geometer.rotation(a)
    Pb, Mb = geometer.position(b), geometer.rotation(b)
    return Ma @ (Pb - Pa), Mb @ Ma.T


def calcTransformations(instrument):
    """Offsets (n-1, 3) and rotation matrices (n-1, 3, 3) between
    consecutive components (acc/run_script.py:141-162)."""
    comps = instrument.components
    offs, rots = [], []
    for i in range(len(comps) - 1):
        o, r = relative_transform(instrument.geometer, comps[i], comps[i + 1])
        offs.append(o)
        rots.append(r)
    return np.array(offs).reshape(-1, 3), np.array(rots).reshape(-1, 3, 3)


def applyTransformation(position, velocity, rotmat, offset):
    """r' = R (r - o), v' = R v on NumPy 3-vectors, in place
    (acc/neutron.py:18-23)."""
    r = rotmat @ (np.asarray(position, dtype=float) - offset)
    v = rotmat @ np.asarray(velocity, dtype=float)
    position[:] = r
    velocity[:] = v
