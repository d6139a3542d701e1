"""Shapes of homogeneous scatterers (the shape objects the reference
renders through acc/geometry/arrow_intersect.py:18-123).  Lengths in m."""

from .shapes import (Block, Box, Cylinder, Difference, HollowCylinder,
                     Intersection, Sphere, Union, epsilon)  # noqa: F401
