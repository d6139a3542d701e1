"""acc/components/optics/guide_anyshape_gravity.py: the mesh guide with
gravity (MCV_OP_GUIDE_ANYSHAPE, ip[2] bit 0); the class lives beside the
mesh guide without gravity."""

from .guide_anyshape import Guide_anyshape_gravity  # noqa: F401

category = 'optics'
