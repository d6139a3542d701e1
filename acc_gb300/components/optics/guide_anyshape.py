"""Guide of arbitrary shape (acc/components/optics/guide_anyshape.py): flat
convex supermirror faces read from an OFF mesh (offio.py), scaled and
centred as the reference does, each packed with its centre, its in-plane
unit vectors and normal, and its polygon in those in-plane coordinates
(include/acc_gb300.h, GUIDE_ANYSHAPE)."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import ComponentBase, set_param

category = 'optics'
max_bounces = 1000
max_numfaces = nat.MCV_ANYSHAPE_MAX_FACES


def load_off(path):
    """(vertices (n, 3), faces (m, k) int) of an OFF file (offio.load,
    acc/components/optics/offio.py:6-28): "OFF", then "nvertices nfaces
    nedges", the vertices, and the faces as "k i1 .. ik", all with the same
    k."""
    with open(path, "rt") as f:
        lines = f.readlines()
    if lines[0].strip() != "OFF":
        raise ValueError(f"{path}: not an OFF file")
    nvertices, nfaces = (int(v) for v in lines[1].split()[:2])
    vertices = np.array([[float(v) for v in lines[2 + i].split()]
                         for i in range(nvertices)])
    faces = []
    for i in range(nfaces):
        numbers = [int(v) for v in lines[2 + nvertices + i].split()]
        if numbers[0] != len(numbers) - 1 or (faces and
                                             len(faces[0]) != numbers[0]):
            raise ValueError(f"{path}: faces must all have the same number "
                             "of vertices")
        faces.append(numbers[1:])
    return vertices, np.array(faces)


def write_off(path, vertices, faces):
    """Write an OFF file of (vertices, faces)."""
    with open(path, "wt") as f:
        f.write("OFF\n%d %d 0\n" % (len(vertices), len(faces)))
        for v in vertices:
            f.write("%r %r %r\n" % tuple(float(x) for x in v))
        for face in faces:
            f.write(" ".join(str(int(i)) for i in [len(face)] + list(face))
                    + "\n")


def box_guide_mesh(w1, h1, w2, h2, l, z0=0.0):
    """(vertices, faces) of a straight or tapering rectangular guide from
    z0 (opening w1 x h1) to z0 + l (w2 x h2), as the reference's example
    meshes order them (tests/components/optics/data/
    guide_anyshape_example1.off): the x = -w/2 wall, the top, the
    x = +w/2 wall, the bottom."""
    a, b = z0, z0 + l
    v = np.array([
        [-w1 / 2, -h1 / 2, a], [-w1 / 2, h1 / 2, a],
        [-w2 / 2, h2 / 2, b], [-w2 / 2, -h2 / 2, b],
        [w1 / 2, -h1 / 2, a], [w1 / 2, h1 / 2, a],
        [w2 / 2, h2 / 2, b], [w2 / 2, -h2 / 2, b]])
    f = np.array([[0, 1, 2, 3], [1, 5, 6, 2], [4, 7, 6, 5], [0, 3, 7, 4]])
    return v, f


def load_scaled_centered_faces(path, xwidth=0, yheight=0, zdepth=0,
                               center=False):
    """The faces (m, k, 3) of an OFF mesh, scaled about the centre of its
    bounding box and optionally centred on the origin
    (guide_anyshape.py:45-85): no size given -> scale 1; one given -> that
    ratio on all axes; all three -> per axis; two -> ValueError."""
    vertices, faces = load_off(path)
    vertices = np.array(vertices, dtype=np.float64)
    lo, hi = vertices.min(axis=0), vertices.max(axis=0)
    c = (lo + hi) / 2
    sizes = (xwidth, yheight, zdepth)
    ratios = [s / (h - l) if s else 0.0 for s, l, h in zip(sizes, lo, hi)]
    given = sum(bool(r) for r in ratios)
    if given == 2:
        raise ValueError("Please provide all of xwidth, yheight, zdepth, or "
                         "none of them, or one of them")
    if given == 1:
        ratios = [sum(ratios)] * 3
    elif given == 0:
        ratios = [1.0] * 3
    for k in range(3):
        vertices[:, k] = ((vertices[:, k] - c[k]) * ratios[k]
                          + (0 if center else c[k]))
    return np.array([[vertices[i] for i in face] for face in faces])


def face_unit_vectors(face):
    """[e1, e2, e3] of a face (guide_anyshape.py:37-43): e1 along its first
    edge, e3 the unit normal of the first two edges, e2 = e3 x e1."""
    seg1, seg2 = face[1] - face[0], face[2] - face[0]
    n = np.cross(seg1, seg2)
    e3 = n / np.linalg.norm(n)
    e1 = seg1 / np.linalg.norm(seg1)
    return np.array([e1, np.cross(e3, e1), e3])


def get_faces_data(geometry, xwidth=0, yheight=0, zdepth=0, center=False):
    """(faces, centers, unitvecs, faces2d) (guide_anyshape.py:160-173):
    centre = mean of a face's vertices, polygon = its vertices in (e1,
    e2)."""
    faces = load_scaled_centered_faces(geometry, xwidth, yheight, zdepth,
                                       center)
    centers = faces.mean(axis=1)
    unitvecs = np.array([face_unit_vectors(f) for f in faces])
    faces2d = np.array([[[np.dot(v - c, e[0]), np.dot(v - c, e[1])]
                         for v in face]
                        for face, c, e in zip(faces, centers, unitvecs)])
    return faces, centers, unitvecs, faces2d


class Guide_anyshape(ComponentBase):
    opcode = nat.OP_GUIDE_ANYSHAPE

    def __init__(self, name, xwidth=0, yheight=0, zdepth=0, center=False,
                 R0=0.99, Qc=0.0219, alpha=3, m=2, W=0.003, geometry="",
                 **kwargs):
        """A guide whose mirrors are the faces of the OFF mesh `geometry`
        (scaled by xwidth / yheight / zdepth and centred when `center`),
        with the supermirror coating R0, Qc, alpha, m, W on every face."""
        self.name = name
        faces, centers, unitvecs, faces2d = get_faces_data(
            geometry, xwidth, yheight, zdepth, center)
        nf, nv = faces2d.shape[:2]
        if not 1 <= nf <= max_numfaces or not 3 <= nv <= \
                nat.MCV_ANYSHAPE_MAX_VERTICES:
            raise ValueError(f"a mesh guide takes 1..{max_numfaces} faces of "
                             f"3..{nat.MCV_ANYSHAPE_MAX_VERTICES} vertices")
        self.propagate_params = (
            faces, centers, unitvecs, faces2d,
            float(R0), float(Qc), float(alpha), float(m), float(W))
        rows = [np.concatenate([c, e[0], e[1], e[2], p.reshape(-1)])
                for c, e, p in zip(centers, unitvecs, faces2d)]
        self.table = np.ascontiguousarray(np.concatenate(rows))

    def pack(self, c, binder):
        faces, centers, unitvecs, faces2d, R0, Qc, alpha, m, W = \
            self.propagate_params
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = faces2d.shape[:2]
        for k, v in enumerate((R0, Qc, alpha, m, W)):
            set_param(c, k, v)
        c.table = binder.table(self, "faces", self.table, np.float64)
        c.ftable = binder.table(self, "faces_f32", self.table, np.float32)
        c.table_len = self.table.size


GRAVITY = 9.80665  # m/s^2 (guide_anyshape_gravity.py:219)


class Guide_anyshape_gravity(Guide_anyshape):
    """Guide_anyshape with gravity (acc/components/optics/
    guide_anyshape_gravity.py): trajectories between reflections are
    parabolas under `gravity`, the acceleration in the guide's own frame
    (by default -9.80665 m/s^2 along y; an instrument sets it from the
    guide's orientation, as the reference's orientation setter does:
    rotation . (0, -9.80665, 0)).  Past its last reflection a neutron short
    of the mesh's largest z is carried to that plane."""

    def __init__(self, name, xwidth=0, yheight=0, zdepth=0, center=False,
                 R0=0.99, Qc=0.0219, alpha=3, m=2, W=0.003, geometry="",
                 gravity=(0.0, -GRAVITY, 0.0), **kwargs):
        super().__init__(name, xwidth, yheight, zdepth, center, R0, Qc,
                         alpha, m, W, geometry)
        if len(self.propagate_params[3]) > 50:
            import warnings
            warnings.warn("with more than 50 faces the reference's list of "
                          "plane hits (100 entries) can overflow, which the "
                          "kernels do not reproduce")
        self.z_max = float(np.max(self.propagate_params[0][:, :, 2]))
        self.gravity = np.asarray(gravity, dtype=np.float64)

    def orient(self, rotation):
        """Set gravity from the guide's rotation in the instrument."""
        self.gravity = np.asarray(rotation, dtype=np.float64) @ \
            np.array([0.0, -GRAVITY, 0.0])

    def pack(self, c, binder):
        super().pack(c, binder)
        c.ip[2] = 1
        for k, v in enumerate(self.gravity):
            set_param(c, 5 + k, float(v))
        set_param(c, 8, self.z_max)
