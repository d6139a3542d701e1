"""Test infrastructure: stand-ins that let the reference's Numba CUDA device
functions run as plain Python on the CPU, so that their outputs on fixed
inputs become golden fixtures.

The reference (mcvine/acc) is Python: every device function is a Python
function under ``@cuda.jit(device=True)``.  Numba, mcni, mccomposite and
mccomponents are not installed here, so this module puts small modules of
those names into ``sys.modules`` before the reference package is imported
as ``mcvine.acc`` (the name its own absolute imports use):

* ``numba.cuda.jit`` returns the Python function unchanged;
  ``cuda.local.array`` is ``numpy.zeros``; ``cuda.atomic.add`` adds in
  place; type objects (``float64``, ``int64``, ``void`` ...) accept the
  signature forms the reference writes (``NB_FLOAT[:]``, ``void(...)``).
* ``xoroshiro128p_uniform_float32(rng_states, threadindex)`` returns the
  next value of ``rng_states``, an injected feed of float32 uniforms (a
  ``Uniforms`` object), so the reference consumes exactly the numbers the
  engine and the oracle consume in their injected-uniform mode.
* Numba types a float32 uniform as float32: ``u * 2`` (float32 with an
  int64) is float64, but ``math.sqrt(u)`` is a float32 square root.  The
  feed returns ``F32`` values that keep those rules (plain float results
  when mixed with other numbers, float32 arithmetic when both operands are
  F32, float32 results from the math functions), and ``FLOAT32_MATH``
  records every math function the reference applied to a float32 value.
* CUDA device math returns NaN/inf where Python's math raises
  (``asin(1.0000001)``, ``sqrt(-0.0)`` is fine, ``log(0)``); the math
  functions that the imported modules hold are replaced with wrappers that
  do the same.
* mcni / mccomposite constants and units: metres, meV, degrees with unit
  value 1 (the reference divides lengths by ``units.length.meter``), and
  the conversion constants of ``acc_gb300.conversion`` (the reference
  imports them from mcni, outside its tree).

Nothing here is imported by the product package; only
``tests/golden/make_reference_fixtures.py`` uses it.
"""

import importlib.abc
import importlib.machinery
import importlib.util
import math
import os
import sys
import types

import numpy as np

FLOAT32_MATH = set()


# ------------------------------------------------------------- float32
class F32(float):
    """A float32 value as Numba types it (see module docstring)."""

    def _bin(self, other, op):
        if isinstance(other, F32):
            return F32(np.float32(op(np.float32(self), np.float32(other))))
        return op(float(self), other)

    def _rbin(self, other, op):
        if isinstance(other, F32):
            return F32(np.float32(op(np.float32(other), np.float32(self))))
        return op(other, float(self))

    def __add__(self, o): return self._bin(o, lambda a, b: a + b)
    def __radd__(self, o): return self._rbin(o, lambda a, b: a + b)
    def __sub__(self, o): return self._bin(o, lambda a, b: a - b)
    def __rsub__(self, o): return self._rbin(o, lambda a, b: a - b)
    def __mul__(self, o): return self._bin(o, lambda a, b: a * b)
    def __rmul__(self, o): return self._rbin(o, lambda a, b: a * b)
    def __truediv__(self, o): return self._bin(o, lambda a, b: a / b)
    def __rtruediv__(self, o): return self._rbin(o, lambda a, b: a / b)
    def __neg__(self): return F32(-float(self))


def _cuda_unary(name, fn):
    def f(x, *rest):
        if isinstance(x, F32) and not rest:
            FLOAT32_MATH.add(name)
            # float32 square root is correctly rounded (IEEE); the other
            # float32 functions are recorded and evaluated the same way
            with np.errstate(all="ignore"):
                return F32(np.float32(getattr(np, _NP.get(name, name))(
                    np.float32(x))))
        try:
            return fn(x, *rest)
        except ValueError:
            return math.nan
        except OverflowError:
            return math.inf
    f.__name__ = name
    return f


_NP = {"asin": "arcsin", "acos": "arccos", "atan": "arctan",
       "atan2": "arctan2", "fabs": "abs"}
_UNARY = ("sqrt", "sin", "cos", "tan", "asin", "acos", "atan", "exp", "log",
          "tanh", "fabs", "log10", "sinh", "cosh")


def _cuda_log(x):
    if x == 0:
        return -math.inf
    if x < 0:
        return math.nan
    return math.log(x)


CUDA_MATH = types.ModuleType("cuda_math")
for _k in dir(math):
    if not _k.startswith("_"):
        setattr(CUDA_MATH, _k, getattr(math, _k))
for _k in _UNARY:
    setattr(CUDA_MATH, _k, _cuda_unary(
        _k, _cuda_log if _k == "log" else getattr(math, _k)))
_ORIG_MATH = {getattr(math, k): getattr(CUDA_MATH, k) for k in _UNARY}


# --------------------------------------------------------------- feeds
class Uniforms:
    """Injected uniforms: one row per neutron, consumed in order."""

    def __init__(self, row):
        self.row = [F32(np.float32(u)) for u in np.asarray(row, np.float32)]
        self.used = 0

    def next(self):
        u = self.row[self.used]
        self.used += 1
        return u


def xoroshiro128p_uniform_float32(rng_states, threadindex):
    return rng_states.next()


# --------------------------------------------------------------- numba
class _NbType:
    def __init__(self, name):
        self.name = name

    def __getitem__(self, item):
        return self

    def __call__(self, *args):
        return ("signature", self.name, args)

    def __repr__(self):
        return f"numba.{self.name}"


def _jit(*args, **kw):
    if len(args) == 1 and callable(args[0]) and not isinstance(
            args[0], _NbType) and not kw:
        return args[0]

    def deco(fn):
        return fn
    return deco


def _local_array(shape, dtype=None):
    name = getattr(dtype, "name", None)
    if dtype is float or dtype is None:
        name = "float64"
    return np.zeros(shape, dtype=np.dtype(name or dtype))


def _atomic_add(arr, idx, val):
    old = arr[idx]
    arr[idx] = old + val
    return old


def _make_module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    m.__path__ = []
    sys.modules[name] = m
    return m


def _install_numba():
    tnames = ("float64", "float32", "int64", "int32", "uint64", "uint32",
              "boolean", "void", "int8", "uint8", "int16")
    typ = {k: _NbType(k) for k in tnames}
    nb = _make_module("numba", __version__="0.58.1", njit=_jit, jit=_jit,
                      vectorize=_jit, guvectorize=_jit, prange=range, **typ)
    cuda = _make_module(
        "numba.cuda", jit=_jit, to_device=lambda a, *x, **k: np.asarray(a),
        is_available=lambda: False, synchronize=lambda: None,
        grid=lambda n: 0 if n == 1 else (0,) * n,
        local=types.SimpleNamespace(array=_local_array),
        const=types.SimpleNamespace(array_like=lambda a: a),
        atomic=types.SimpleNamespace(add=_atomic_add),
        # libdevice's double functions: sqrt/floor/fabs are exact, sin/cos
        # to within an ulp of the host's
        libdevice=types.SimpleNamespace(
            sqrt=lambda x: CUDA_MATH.sqrt(x), sin=lambda x: CUDA_MATH.sin(x),
            cos=lambda x: CUDA_MATH.cos(x), fabs=lambda x: CUDA_MATH.fabs(x),
            floor=math.floor),
        device_array=lambda shape, dtype=float: np.zeros(shape, dtype),
        **typ)
    rnd = _make_module(
        "numba.cuda.random",
        xoroshiro128p_uniform_float32=xoroshiro128p_uniform_float32,
        xoroshiro128p_type=_NbType("xoroshiro128p_type"),
        create_xoroshiro128p_states=lambda n, seed=0: None)
    cuda.random = rnd
    nb.cuda = cuda
    core = _make_module("numba.core")
    core.config = _make_module("numba.core.config", ENABLE_CUDASIM=False)

    class Array:  # noqa: D401 - type placeholders
        pass

    class Float:
        pass
    core.types = _make_module("numba.core.types", Array=Array, Float=Float,
                              **typ)
    nb.core = core
    nb.types = core.types


# -------------------------------------------------- mcni and relatives
class _Dummy:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Dummy()

    def __setitem__(self, k, v):
        pass

    def __getitem__(self, k):
        return _Dummy()


class _AutoModule(types.ModuleType):
    """A module whose unknown attributes are placeholder classes."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        cls = type(name, (_Dummy,), {})
        setattr(self, name, cls)
        return cls


class _AutoFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    ROOTS = ("mcni", "mccomposite", "mccomponents", "histogram",
             "sampleassembly", "instrument", "danse", "pyre", "journal")

    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in self.ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self,
                                                  is_package=True)
        return None

    def create_module(self, spec):
        m = _AutoModule(spec.name)
        m.__path__ = []
        return m

    def exec_module(self, module):
        pass


def _install_mcni():
    from acc_gb300 import conversion as C
    if not any(isinstance(f, _AutoFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _AutoFinder())
    units = types.SimpleNamespace(
        length=types.SimpleNamespace(meter=1.0, m=1.0, angstrom=1e-10,
                                     cm=1e-2, mm=1e-3),
        energy=types.SimpleNamespace(meV=1.0, eV=1e3),
        angle=types.SimpleNamespace(degree=1.0, deg=1.0),
        time=types.SimpleNamespace(second=1.0, s=1.0))
    import mcni  # noqa: F401  (auto module)
    import mcni.utils  # noqa: F401
    conv = sys.modules["mcni.utils"].conversion = _make_module(
        "mcni.utils.conversion", V2K=C.V2K, K2V=C.K2V, SE2V=C.SE2V,
        VS2E=C.VS2E, v2e=C.v2e, e2v=C.e2v, v2k=C.v2k, k2v=C.k2v)
    sys.modules["mcni"].units = units
    sys.modules["mcni"].utils = sys.modules["mcni.utils"]
    sys.modules["mcni.utils"].conversion = conv
    sys.modules["mcni.units"] = units
    import mccomposite  # noqa: F401
    import mccomposite.units_utils  # noqa: F401

    class UnitsRemover:
        def __init__(self, length_unit=1.0, angle_unit=1.0):
            pass

        def remove_unit(self, x, unit):
            # the kernel descriptions here hold plain numbers already in
            # the unit asked for (mccomposite divides quantities by it)
            return x
    sys.modules["mccomposite.units_utils"].UnitsRemover = UnitsRemover
    sys.modules["mccomposite"].units = units


# ---------------------------------------------------- the reference package
def load_reference(root):
    """Import the reference's ``acc`` package (under ``root``) as
    ``mcvine.acc`` with the stand-ins installed; returns the package."""
    if "mcvine.acc" in sys.modules:
        return sys.modules["mcvine.acc"]
    os.environ.pop("NUMBA_ENABLE_CUDASIM", None)
    _install_numba()
    _install_mcni()
    acc_dir = os.path.join(root, "acc")
    mcvine = _make_module("mcvine")
    spec = importlib.util.spec_from_file_location(
        "mcvine.acc", os.path.join(acc_dir, "__init__.py"),
        submodule_search_locations=[acc_dir])
    acc = importlib.util.module_from_spec(spec)
    sys.modules["mcvine.acc"] = acc
    spec.loader.exec_module(acc)
    mcvine.acc = acc
    return acc


def import_ref(name):
    """Import ``mcvine.acc.<name>`` and route its math through CUDA_MATH."""
    mod = importlib.import_module("mcvine.acc." + name)
    patch_math()
    return mod


def patch_math():
    """Point every imported reference module's math names at CUDA_MATH."""
    for k, m in list(sys.modules.items()):
        if not k.startswith("mcvine.acc") or m is None:
            continue
        d = m.__dict__
        for attr, val in list(d.items()):
            if val is math:
                d[attr] = CUDA_MATH
            elif callable(val) and not isinstance(val, type):
                try:
                    rep = _ORIG_MATH.get(val)
                except TypeError:
                    rep = None
                if rep is not None:
                    d[attr] = rep
