"""Sample assemblies: the XML files that instrument scripts hand to
loadFirstHomogeneousScatterer (acc/components/samples/__init__.py:1-48).

The reference reads them through mcvine's sampleassembly and mccomponents
packages (outside its tree).  This module reads the subset its sample
scripts use (tests/components/samples/sampleassemblies):

* sampleassembly.xml: <SampleAssembly> with scatterers (<PowderSample>,
  <SingleCrystal>, <Sample> ...) that each hold a <Shape> (sphere, cylinder,
  block and their difference / union / intersection) and a <Phase> (a
  chemical formula and an xyz file of the unit cell);
* <name>-scatterer.xml beside it: a <homogeneous_scatterer> whose kernel is
  an IsotropicKernel, E_Q_Kernel, ConstantQEKernel,
  SimplePowderDiffractionKernel (peaks from a peaks.py or a .laz file),
  SANS2D_ongrid_Kernel, DGSSXResKernel, or a KernelContainer of them.  When
  several kernels stand side by side the last one is the scatterer's.

Attribute values are unit expressions ("1*cm", "10./m", "3/angstrom",
"30*meV", "2.*millisecond + 1.*millisecond"), evaluated with a fixed table
of units and nothing else.  A kernel without absorption / scattering
coefficients takes them from its scatterer's unit cell: the sums of the
atoms' absorption (at 2200 m/s) and coherent + incoherent cross sections
over the cell volume (1 barn / A^3 = 100 / m), the cross sections taken
from the table below (values of the NIST neutron scattering length
tables).
"""

import ast
import math
import os
import xml.etree.ElementTree as ET
from collections import namedtuple

import numpy as np

# units in metres, seconds, meV, degrees
UNITS = {
    "m": 1.0, "meter": 1.0, "meters": 1.0, "cm": 1e-2, "mm": 1e-3,
    "um": 1e-6, "micron": 1e-6, "nm": 1e-9, "angstrom": 1e-10,
    "inch": 0.0254, "s": 1.0, "second": 1.0, "ms": 1e-3,
    "millisecond": 1e-3, "us": 1e-6, "microsecond": 1e-6, "meV": 1.0,
    "eV": 1e3, "deg": 1.0, "degree": 1.0, "K": 1.0, "barn": 1e-28,
}

# per-atom (coherent, incoherent, absorption at 2200 m/s) cross sections,
# barn
CROSS_SECTIONS = {
    "H": (1.7568, 80.26, 0.3326),
    "C": (5.551, 0.001, 0.0035),
    "N": (11.01, 0.5, 1.9),
    "O": (4.232, 0.0008, 0.00019),
    "Al": (1.495, 0.0082, 0.231),
    "Si": (2.163, 0.004, 0.171),
    "V": (0.0184, 5.08, 5.08),
    "Fe": (11.22, 0.4, 2.56),
    "Ni": (13.3, 5.2, 4.49),
    "Cu": (7.485, 0.55, 3.78),
    "U": (8.903, 0.005, 7.57),
}

_ALLOWED = (ast.Expression, ast.BinOp, ast.UnaryOp, ast.Constant, ast.Name,
            ast.Load, ast.Add, ast.Sub, ast.Mult, ast.Div, ast.Pow,
            ast.USub, ast.UAdd, ast.Tuple)


def quantity(text, unit=1.0):
    """The value of a unit expression in `unit` (a UNITS value, or a
    product / quotient of them): quantity("1*cm", UNITS["m"]) = 0.01,
    quantity("10./m", 1 / UNITS["m"]) = 10.  A plain number is taken to be
    in `unit` already.  A comma-separated list gives a tuple."""
    text = str(text).strip()
    tree = ast.parse(text, mode="eval")
    for node in ast.walk(tree):
        if not isinstance(node, _ALLOWED):
            raise ValueError(f"not a unit expression: {text!r}")
        if isinstance(node, ast.Name) and node.id not in UNITS:
            raise ValueError(f"unknown unit {node.id!r} in {text!r}")
    has_units = any(isinstance(n, ast.Name) for n in ast.walk(tree))
    v = eval(compile(tree, "<units>", "eval"), {"__builtins__": {}},
             dict(UNITS))
    scale = unit if has_units else 1.0
    if isinstance(v, tuple):
        return tuple(float(x) / scale for x in v)
    return float(v) / scale


# ------------------------------------------------------------ unit cells
UnitCell = namedtuple("UnitCell", "lattice atoms volume")


def read_xyz(path):
    """An xyz file (natoms; nine lattice-vector components in A; one
    'Element x y z' row per atom, fractional coordinates)."""
    with open(path) as f:
        rows = [ln.split() for ln in f if ln.strip()]
    n = int(rows[0][0])
    lattice = np.array([float(v) for v in rows[1][:9]]).reshape(3, 3)
    atoms = [(r[0], tuple(float(v) for v in r[1:4])) for r in rows[2:2 + n]]
    if len(atoms) != n:
        raise ValueError(f"{path}: {n} atoms announced, {len(atoms)} read")
    return UnitCell(lattice, atoms, abs(float(np.linalg.det(lattice))))


def cell_coefficients(cell):
    """(absorption coefficient at 2200 m/s, scattering coefficient), 1/m,
    of a unit cell: per-cell cross sections (barn) / volume (A^3) x 100."""
    sabs = sscat = 0.0
    for el, _ in cell.atoms:
        if el not in CROSS_SECTIONS:
            raise KeyError(f"no cross sections for element {el!r}; give the "
                           "kernel absorption_coefficient and "
                           "scattering_coefficient")
        coh, inc, ab = CROSS_SECTIONS[el]
        sabs += ab
        sscat += coh + inc
    return sabs / cell.volume * 100.0, sscat / cell.volume * 100.0


# ------------------------------------------------------------ powder peaks
def read_laz(path, debye_waller=1.0):
    """Peaks of a Lazy-format (.laz) file: one reflection a row, the
    multiplicity, d spacing and |F| in the columns its '# column_j',
    '# column_d' and '# column_F' header lines name (1-based); q = 2 pi / d,
    F^2 = |F|^2.  Returns (peaks, unit cell volume A^3, per-cell (coh, inc,
    abs) cross sections from the sigma_* and nb_atoms header lines)."""
    from .kernels import Peak
    cols = {"j": 17, "d": 6, "F": 13}
    head = {}
    cell = None
    peaks = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s:
                continue
            if s.startswith("#"):
                w = s[1:].split()
                if len(w) >= 2 and w[0] in ("column_j", "column_d",
                                            "column_F"):
                    cols[w[0][-1]] = int(w[1])
                elif len(w) >= 2 and w[0] in ("sigma_coh", "sigma_inc",
                                              "sigma_abs", "nb_atoms"):
                    head[w[0]] = float(w[1])
                elif len(w) >= 7 and w[0] == "CELL":
                    cell = [float(v) for v in w[1:7]]
                continue
            v = s.split()
            d = float(v[cols["d"] - 1])
            F = float(v[cols["F"] - 1])
            j = int(float(v[cols["j"] - 1]))
            peaks.append(Peak(q=2 * math.pi / d, F_squared=F * F,
                              multiplicity=j,
                              DebyeWaller_factor=debye_waller,
                              intrinsic_line_width=0.0))
    if cell is None:
        raise ValueError(f"{path}: no '# CELL' line")
    a, b, c = cell[:3]
    al, be, ga = (math.radians(x) for x in cell[3:])
    vol = a * b * c * math.sqrt(
        1 - math.cos(al) ** 2 - math.cos(be) ** 2 - math.cos(ga) ** 2
        + 2 * math.cos(al) * math.cos(be) * math.cos(ga))
    n = head.get("nb_atoms", 1.0)
    xs = (n * head.get("sigma_coh", 0.0), n * head.get("sigma_inc", 0.0),
          n * head.get("sigma_abs", 0.0))
    return sorted(peaks, key=lambda p: p.q), vol, xs


def read_peaks_py(path):
    """Peaks of a peaks.py file: the module defines `peaks` (Peak(q=...,
    F_squared=..., multiplicity=..., intrinsic_line_width=...,
    DebyeWaller_factor=...)), `unitcell_volume` and a `cross_sections`
    namespace (coh, inc, abs per cell, barn).  It is run with Peak taken
    from this package in place of mccomponents'."""
    import sys
    import types
    from .kernels import Peak
    name = "mccomponents.sample.diffraction.SimplePowderDiffractionKernel"
    saved = {k: sys.modules.get(k) for k in
             ("mccomponents", "mccomponents.sample",
              "mccomponents.sample.diffraction", name)}
    try:
        for k in saved:
            if saved[k] is None:
                sys.modules[k] = types.ModuleType(k)
        sys.modules[name].Peak = Peak
        ns = {"__file__": path, "__name__": "peaks"}
        with open(path) as f:
            exec(compile(f.read(), path, "exec"), ns)
    finally:
        for k, m in saved.items():
            if m is None:
                sys.modules.pop(k, None)
    xs = ns["cross_sections"]
    return (sorted(ns["peaks"], key=lambda p: p.q),
            float(ns["unitcell_volume"]),
            (float(xs.coh), float(xs.inc), float(xs.abs)))


# ---------------------------------------------------------------- shapes
def _shape(el):
    from .geometry import Block, Cylinder, Difference, Intersection, \
        Sphere, Union
    tag = el.tag.lower()
    m = UNITS["m"]
    if tag == "sphere":
        return Sphere(quantity(el.get("radius"), m))
    if tag == "cylinder":
        return Cylinder(quantity(el.get("radius"), m),
                        quantity(el.get("height"), m))
    if tag == "block":
        return Block(quantity(el.get("width"), m),
                     quantity(el.get("height"), m),
                     quantity(el.get("thickness"), m))
    ops = {"difference": Difference, "union": Union,
           "intersection": Intersection}
    if tag in ops:
        kids = [k for k in el if isinstance(k.tag, str)]
        if len(kids) != 2:
            raise ValueError(f"<{el.tag}> needs two shapes")
        return ops[tag](_shape(kids[0]), _shape(kids[1]))
    raise ValueError(f"shape <{el.tag}> is not supported")


# --------------------------------------------------------------- kernels
def _coefficients(el, cell):
    mu = el.get("absorption_coefficient")
    sigma = el.get("scattering_coefficient")
    if mu is not None and sigma is not None:
        inv_m = 1.0 / UNITS["m"]
        return quantity(mu, inv_m), quantity(sigma, inv_m)
    if cell is None:
        raise ValueError(f"<{el.tag}> has no absorption / scattering "
                         "coefficients and its scatterer no unit cell")
    return cell_coefficients(cell)


def _kernel(el, cell, directory):
    from . import kernels as K
    tag = el.tag
    inv_A = 1.0 / UNITS["angstrom"]
    if tag == "KernelContainer":
        kids = [_kernel(k, cell, directory) for k in el
                if isinstance(k.tag, str)]
        for k, x in zip(kids, [k for k in el if isinstance(k.tag, str)]):
            if x.get("weight") is not None:
                k.weight = float(quantity(x.get("weight")))
        avg = str(el.get("average", "no")).lower() in ("yes", "true", "1")
        return K.CompositeKernel(kids, average=avg)
    if tag == "IsotropicKernel":
        return K.IsotropicKernel(*_coefficients(el, cell))
    if tag == "E_Q_Kernel":
        mu, sigma = _coefficients(el, cell)
        return K.E_Q_Kernel(el.get("E_Q"), el.get("S_Q"),
                            quantity(el.get("Qmin"), inv_A),
                            quantity(el.get("Qmax"), inv_A), mu, sigma)
    if tag == "ConstantQEKernel":
        mu, sigma = _coefficients(el, cell)
        return K.ConstantQEKernel(
            quantity(el.get("momentum-transfer"), inv_A),
            quantity(el.get("energy-transfer"), UNITS["meV"]), mu, sigma)
    if tag == "SimplePowderDiffractionKernel":
        dw = float(quantity(el.get("DebyeWaller_factor", "1")))
        if el.get("peaks-py-path"):
            peaks, vol, xs = read_peaks_py(
                os.path.join(directory, el.get("peaks-py-path")))
        elif el.get("laz-path"):
            peaks, vol, xs = read_laz(
                os.path.join(directory, el.get("laz-path")), dw)
        else:
            raise ValueError("SimplePowderDiffractionKernel needs a "
                             "peaks-py-path or a laz-path")
        coh, inc, ab = xs
        return K.SimplePowderDiffractionKernel(
            peaks, vol, absorption_cross_section=ab,
            incoherent_cross_section=inc, coherent_cross_section=coh)
    if tag == "SANS2D_ongrid_Kernel":
        mu, sigma = _coefficients(el, cell)
        return K.SANS2D_ongrid_Kernel(
            os.path.join(directory, el.get("S_QxQy")),
            quantity(el.get("Qx_min"), inv_A),
            quantity(el.get("Qx_max"), inv_A),
            quantity(el.get("Qy_min"), inv_A),
            quantity(el.get("Qy_max"), inv_A), mu, sigma)
    if tag == "DGSSXResKernel":
        mu, sigma = _coefficients(el, cell)
        return K.DGSSXResKernel(
            quantity(el.get("target-position"), UNITS["m"]),
            quantity(el.get("target-radius"), UNITS["m"]),
            quantity(el.get("tof-at-target"), UNITS["s"]),
            quantity(el.get("dtof"), UNITS["s"]), mu, sigma)
    raise ValueError(f"kernel <{tag}> is not supported")


# ------------------------------------------------------------- scatterers
class HomogeneousScatterer:
    """One scatterer of an assembly: shape() and kernel() as in mcvine's
    homogeneous scatterer, plus its name and unit cell."""

    def __init__(self, name, shape, kernel, cell=None, attributes=None):
        self.name = name
        self._shape = shape
        self._kernel = kernel
        self.cell = cell
        self.attributes = dict(attributes or {})

    def shape(self):
        return self._shape

    def kernel(self):
        return self._kernel


class ScattererComposite:
    """The scatterers of an assembly, in file order (elements())."""

    def __init__(self, name, scatterers, attributes=None):
        self.name = name
        self._elements = list(scatterers)
        self.attributes = dict(attributes or {})

    def elements(self):
        return list(self._elements)


_SCATTERER_TAGS = ("PowderSample", "SingleCrystal", "Sample", "Scatterer",
                   "Container", "Environment")


def load(sampleassembly_xml):
    """Read a sample assembly: ScattererComposite of HomogeneousScatterer
    (each scatterer's kernel from <name>-scatterer.xml beside the file)."""
    path = os.path.realpath(sampleassembly_xml)
    directory = os.path.dirname(path)
    root = ET.parse(path).getroot()
    scatterers = []
    for el in root:
        if not isinstance(el.tag, str) or el.tag not in _SCATTERER_TAGS:
            continue
        name = el.get("name")
        shape_el = el.find("Shape")
        if shape_el is None:
            raise ValueError(f"scatterer {name!r} has no <Shape>")
        kids = [k for k in shape_el if isinstance(k.tag, str)]
        if len(kids) != 1:
            raise ValueError(f"<Shape> of {name!r} needs one shape")
        shape = _shape(kids[0])
        cell = None
        phase = el.find("Phase")
        if phase is not None and phase.find("xyzfile") is not None:
            xyz = os.path.join(directory, phase.find("xyzfile").text.strip())
            if os.path.exists(xyz):
                cell = read_xyz(xyz)
        sc_path = os.path.join(directory, f"{name}-scatterer.xml")
        kernel = None
        sc_attrs = {}
        if os.path.exists(sc_path):
            sc = ET.parse(sc_path).getroot()
            sc_attrs = dict(sc.attrib)
            for k in sc:
                if isinstance(k.tag, str):
                    kernel = _kernel(k, cell, directory)
        scatterers.append(HomogeneousScatterer(name, shape, kernel, cell,
                                               sc_attrs))
    return ScattererComposite(root.get("name"), scatterers,
                              dict(root.attrib))
