"""Shape descriptions packed into an HSS component.

A shape is a primitive (sphere, cylinder with its axis along local z, box)
or one binary CSG node (difference, union, intersection) over two
primitives, the cases arrow_intersect.py:28-123 renders for the samples in
scope.  Deeper CSG trees are not supported.
"""

from .. import _native as nat

epsilon = 1e-10  # acc/geometry/__init__.py:2


class Shape:
    def identify(self, visitor):
        return getattr(visitor, "on" + type(self).__name__)(self)


class Primitive(Shape):
    kind = 0

    def params(self):
        raise NotImplementedError


class Sphere(Primitive):
    kind = nat.SHAPE_SPHERE

    def __init__(self, radius):
        self.radius = float(radius)

    def params(self):
        return (self.radius, 0.0, 0.0)


class Cylinder(Primitive):
    """x^2 + y^2 <= radius^2, |z| <= height/2 (arrow_intersect.py:171-177)."""
    kind = nat.SHAPE_CYLINDER

    def __init__(self, radius, height):
        self.radius = float(radius)
        self.height = float(height)

    def params(self):
        return (self.radius, self.height, 0.0)


class Block(Primitive):
    """width (x) x height (y) x thickness (z) box centred at the origin."""
    kind = nat.SHAPE_BOX

    def __init__(self, width, height, thickness):
        self.width = float(width)
        self.height = float(height)
        self.thickness = float(thickness)

    def params(self):
        return (self.width, self.height, self.thickness)


Box = Block


class Binary(Shape):
    op = 0

    def __init__(self, op1, op2):
        if not (isinstance(op1, Primitive) and isinstance(op2, Primitive)):
            raise NotImplementedError(
                "CSG nodes over primitives only (one level)")
        self.op1, self.op2 = op1, op2

    @property
    def shapes(self):
        return (self.op1, self.op2)


class Difference(Binary):
    op = nat.CSG_DIFFERENCE


class Union(Binary):
    op = nat.CSG_UNION


class Intersection(Binary):
    op = nat.CSG_INTERSECTION


def HollowCylinder(in_radius, out_radius, height):
    """Difference of two coaxial cylinders; the inner one is 10% taller so
    that no cap is shared (as tests/geometry/hollowcylinder_example1.xml:5-8
    builds it)."""
    return Difference(Cylinder(out_radius, height),
                      Cylinder(in_radius, 1.1 * height))


def pack_shape(shape, c, set_param):
    """Fill ip[0] (CSG op), ip[2], ip[3] (primitive kinds), dp[0:3], dp[4:7]."""
    if isinstance(shape, Primitive):
        c.ip[0] = nat.CSG_PRIMITIVE
        c.ip[2] = shape.kind
        for k, v in enumerate(shape.params()):
            set_param(c, k, v)
    elif isinstance(shape, Binary):
        c.ip[0] = shape.op
        c.ip[2] = shape.op1.kind
        c.ip[3] = shape.op2.kind
        for k, v in enumerate(shape.op1.params()):
            set_param(c, k, v)
        for k, v in enumerate(shape.op2.params()):
            set_param(c, 4 + k, v)
    else:
        raise TypeError(f"not a shape: {shape!r}")
