"""Test infrastructure: run the reference's own device functions (Python
under Numba decorators) on the CPU for the cases of ``reference_cases.py``
and write their outputs to ``reference_paths.npz`` beside this script.

    python tests/golden/make_reference_fixtures.py [REFERENCE_ROOT]

REFERENCE_ROOT is the mcvine/acc source tree (the directory holding
``acc/``); it defaults to $MCVINE_ACC_REFERENCE, then /root/reference.
The stand-ins for numba / mcni are in ``refshim.py``.

Per case the file holds ``<case>.in`` (input neutrons; absent for a
source), ``<case>.u`` (float32 uniforms, one row per neutron),
``<case>.out`` (the neutron after the reference's ``propagate``),
``<case>.used`` (uniforms consumed), ``<case>.valid`` (False where the
reference's Python raised: such neutrons are left out of the comparison)
and, for monitors, ``<case>.hist`` (the reference's ``out`` array).

Two readings are applied to the reference before it runs:

* ``cu_device_intersect_cylinder`` (acc/geometry/arrow_intersect.py:241-267)
  returns nothing when a ray misses the cylinder (``if n==0: np.nan,
  np.nan`` lacks its ``return``); it is read as returning (nan, nan), a
  miss, which is what the statement spells;
* ``SNS_source.__init__`` calls ``warnings.warn`` for a disc face
  (acc/components/sources/SNS_source.py:129) in a module that never imports
  ``warnings``; the module is given it.
"""

import json
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [HERE, ROOT]

import refshim  # noqa: E402
import reference_cases as RC  # noqa: E402


class _Kernel:
    """A kernel description with the attributes the reference's
    ScatterFuncFactory reads (acc/kernels/__init__.py)."""

    def __init__(self, visit, **attrs):
        self._visit = visit
        self.__dict__.update(attrs)

    def identify(self, visitor):
        return getattr(visitor, self._visit)(self)


def ref_kernel(k):
    kind = k["kind"]
    if kind == "isotropic":
        return _Kernel("onIsotropicKernel", absorption_coefficient=k["mu"],
                       scattering_coefficient=k["sigma"])
    if kind == "powder":
        peaks = [types.SimpleNamespace(**p) for p in k["peaks"]]
        V = k["unitcell_volume"]
        # the sample assembly's coefficients: per-cell cross sections over
        # the cell volume, barn/A^3 -> 1/m
        return _Kernel(
            "onSimplePowderDiffractionKernel", peaks=peaks,
            unitcell_volume=V,
            cross_sections=types.SimpleNamespace(abs=k["abs"], inc=k["inc"],
                                                 coh=k["coh"]),
            absorption_coefficient=k["abs"] / V * 100,
            scattering_coefficient=(k["inc"] + k["coh"]) / V * 100)
    if kind == "E_Q":
        return _Kernel("onE_Q_Kernel", E_Q=k["E_Q"], S_Q=k["S_Q"],
                       Qmin=k["Qmin"], Qmax=k["Qmax"],
                       absorption_coefficient=k["mu"],
                       scattering_coefficient=k["sigma"])
    if kind == "constant_qe":
        return _Kernel("onConstantQEKernel", Q=k["Q"], E=k["E"],
                       absorption_coefficient=k["mu"],
                       scattering_coefficient=k["sigma"])
    raise ValueError(kind)


def main(root):
    refshim.load_reference(root)
    imp = refshim.import_ref
    cb = imp("components.ComponentBase")
    # constructors send one neutron through `process` to trigger Numba's
    # compilation; there is nothing to compile here
    cb.ComponentBase.process = lambda self, neutrons: neutrons
    ai = imp("geometry.arrow_intersect")
    _cyl = ai.cu_device_intersect_cylinder

    def cylinder_or_miss(*a):
        r = _cyl(*a)
        return (math.nan, math.nan) if r is None else r
    ai.cu_device_intersect_cylinder = cylinder_or_miss
    src = imp("components.sources.source_simple")
    guide = imp("components.optics.guide")
    sns = imp("components.sources.SNS_source")
    sts = imp("components.sources.STS_source")
    # SNS_source.__init__ warns on a disc face (SNS_source.py:129) without
    # importing `warnings`; the module gets it here so that the disc can run
    import warnings
    sns.warnings = warnings
    hss = imp("components.samples.homogeneous_single_scatterer")
    mons = {k: imp("components.monitors." + k) for k in
            ("psd_monitor", "wavelength_monitor", "psd_monitor_4pi",
             "iqe_monitor")}
    classes = {"psd_monitor": "PSD_monitor",
               "wavelength_monitor": "Wavelength_monitor",
               "psd_monitor_4pi": "PSD_monitor_4Pi",
               "iqe_monitor": "IQE_monitor"}
    refshim.patch_math()

    arrays, meta = {}, {}
    for ci, (name, case) in enumerate(RC.CASES.items()):
        kind = case["kind"]
        seed = 100 + ci
        inp = RC.draw_inputs(case, seed)
        u = RC.draw_uniforms(case, seed)
        n = case["n"]
        hist = None
        if kind == "source":
            comp = src.Source_simple(name, **case["kw"])

            def call(nt, feed, comp=comp):
                src.Source_simple.propagate(0, feed, nt,
                                            *comp.propagate_params)
        elif kind in ("sns_source", "sts_source"):
            import warnings
            mod = sns if kind == "sns_source" else sts
            cls = mod.SNS_source if kind == "sns_source" else mod.STS_source
            path = os.path.join(root, "tests", "components", "sources",
                                case["file"])
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                comp = cls(name, path, **case["kw"])
            refshim.patch_math()

            def call(nt, feed, comp=comp, cls=cls):
                cls.propagate(0, feed, nt, *comp.propagate_params)
        elif kind == "guide":
            comp = guide.Guide(name, **case["kw"])

            def call(nt, feed, comp=comp):
                guide.Guide.propagate(nt, *comp.propagate_params)
        elif kind == "hss":
            cls = hss.factory(shape=RC._product_shape(case["shape"]),
                              kernel=ref_kernel(case["kernel"]))
            refshim.patch_math()

            def call(nt, feed, cls=cls):
                cls.propagate(0, feed, nt)
        else:
            mcls = getattr(mons[kind], classes[kind])
            comp = mcls(name, **case["kw"])
            hist = comp.out

            def call(nt, feed, comp=comp, mcls=mcls):
                mcls.propagate(nt, *comp.propagate_params)
        out = np.full((n, 10), np.nan)
        used = np.zeros(n, np.int32)
        valid = np.ones(n, bool)
        errors = {}
        for i in range(n):
            nt = np.zeros(10) if inp is None else inp[i].copy()
            feed = refshim.Uniforms(u[i])
            try:
                call(nt, feed)
            except (ZeroDivisionError, TypeError, IndexError) as e:
                valid[i] = False
                errors[type(e).__name__] = errors.get(type(e).__name__, 0) + 1
                continue
            out[i] = nt
            used[i] = feed.used
        assert used.max() <= u.shape[1], (name, used.max())
        if inp is not None:
            arrays[name + ".in"] = inp
        arrays[name + ".u"] = u
        arrays[name + ".out"] = out
        arrays[name + ".used"] = used
        arrays[name + ".valid"] = valid
        if hist is not None:
            arrays[name + ".hist"] = np.array(hist)
        meta[name] = dict(invalid=int((~valid).sum()), errors=errors,
                          absorbed=int((out[valid, 9] <= 0).sum()),
                          max_uniforms=int(used.max()))
        print(name, meta[name])
    meta["_float32_math"] = sorted(refshim.FLOAT32_MATH)
    print("float32 math in the reference:", meta["_float32_math"])
    np.savez_compressed(os.path.join(HERE, "reference_paths.npz"), **arrays)
    with open(os.path.join(HERE, "reference_paths.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    root = (sys.argv[1] if len(sys.argv) > 1 else
            os.environ.get("MCVINE_ACC_REFERENCE", "/root/reference"))
    main(root)
