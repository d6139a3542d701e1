"""Beamstop: absorb neutrons that hit a rectangle or disc at z=0
(acc/components/optics/beamstop.py:17-112)."""

from ... import _native as nat
from .slit import Slit

category = 'optics'


class Beamstop(Slit):
    opcode = nat.OP_BEAMSTOP
    _kind = "beamstop"
