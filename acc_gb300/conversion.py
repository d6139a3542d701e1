"""Neutron unit conversions.

The reference imports these from mcni.utils.conversion (outside the
reference tree; V2K appears in acc/components/optics/guide_baseline.py:16-17).
The values are the McStas/mcni definitions: v [m/s], k [1/A], E [meV].
"""
import math

V2K = 1.58825361e-3
K2V = 1.0 / V2K
SE2V = 437.393377
VS2E = 5.22703725e-6


def v2e(v):
    return v * v * VS2E


def e2v(e):
    return math.sqrt(e) * SE2V


def v2k(v):
    return v * V2K


def k2v(k):
    return k * K2V
