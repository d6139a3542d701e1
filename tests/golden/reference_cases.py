"""Test infrastructure: the per-component cases whose outputs come from the
reference's own device functions (``make_reference_fixtures.py`` runs them
on the CPU and writes ``reference_paths.npz``).

Each case names a component, its constructor arguments, how its input
neutrons are drawn (seeded) and how many float32 uniforms each neutron
gets.  ``build_product(case)`` makes the same component from this package,
so that a test can run it through the oracle and through the GPU engine in
their injected-uniform mode and compare with the reference's outputs.
"""

import math

import numpy as np

from acc_gb300.conversion import SE2V

# config 5's 50 peaks (d uniform 0.5-4 A, F^2 lognormal(0, 1),
# multiplicity in {2,4,6,8,12,24}, Debye-Waller exp(-0.005/d^2)), plus a
# line width on half of them in the broadened case
def powder_peak_rows(npeaks=50, seed=0, width=0.0):
    rng = np.random.default_rng(seed)
    d = rng.uniform(0.5, 4.0, npeaks)
    F2 = rng.lognormal(0.0, 1.0, npeaks)
    mult = rng.choice([2, 4, 6, 8, 12, 24], npeaks)
    w = np.where(np.arange(npeaks) % 2 == 0, width, 0.0)
    rows = sorted(((2 * math.pi / di, f, int(m), math.exp(-0.005 / di ** 2),
                    float(wi)) for di, f, m, wi in zip(d, F2, mult, w)))
    return [dict(q=q, F_squared=f, multiplicity=m, DebyeWaller_factor=dw,
                 intrinsic_line_width=wi) for q, f, m, dw, wi in rows]


# the reference's Al powder sample
# (tests/components/samples/sampleassemblies/Al-simplepowderdiffractionkernel/peaks.py):
# two peaks, DW factor 0 (taken as 1), a = 4.04932 A, 4 atoms
AL_A = 4.049320
AL_PEAKS = [dict(q=1.9200, F_squared=0.0, multiplicity=12,
                 intrinsic_line_width=0, DebyeWaller_factor=0),
            dict(q=3.1353, F_squared=3.3, multiplicity=8,
                 intrinsic_line_width=0, DebyeWaller_factor=0)]
AL_XS = dict(coh=4 * 1.495, inc=4 * 0.0082, abs=4 * 0.231)

# the reference's moderator files (tests/components/sources), shipped
# gzip-compressed in acc_gb300/data
SNS_FILE = "source_rot2_cdr_cyl_3x3_20190417.dat"
STS_FILE = "BL20-CY-123D-STS-Min-2G-source_mctal-195_sp.dat"


def moderator_path(name):
    """The package's copy of a reference moderator file."""
    from acc_gb300.instruments import shipped_moderator
    return shipped_moderator(name)


GUIDE_COATING = dict(R0=0.99, Qc=0.0219, alpha=3.0, m=3.0, W=0.003)

CASES = {
    # Source_simple (acc/components/sources/source_simple.py:47-162)
    "source_disc_config1": dict(
        kind="source", n=256, nu=5,
        kw=dict(radius=0.05, dist=5.0, xw=0.01, yh=0.01, E0=60.0, dE=10.0)),
    "source_disc_guide": dict(
        kind="source", n=256, nu=5,
        kw=dict(radius=0.05, dist=1.0, xw=0.05, yh=0.05, E0=52.5,
                dE=47.5)),
    "source_square_wavelength": dict(
        kind="source", n=256, nu=5,
        kw=dict(radius=0, width=0.03, height=0.02, dist=2.0, xw=0.04,
                yh=0.02, E0=0, dE=0, Lambda0=2.0, dLambda=0.5, flux=3.0,
                N=7)),
    # Guide (acc/components/optics/guide.py:23-162)
    "guide_straight": dict(
        kind="guide", n=256, nu=1, inputs="guide",
        kw=dict(w1=0.05, h1=0.05, w2=0.05, h2=0.05, l=10.0,
                **GUIDE_COATING)),
    "guide_tapered": dict(
        kind="guide", n=256, nu=1, inputs="guide",
        kw=dict(w1=0.05, h1=0.05, w2=0.02, h2=0.02, l=5.0,
                **GUIDE_COATING)),
    "guide_mixed_taper_defaults": dict(
        kind="guide", n=256, nu=1, inputs="guide",
        kw=dict(w1=0.03, h1=0.04, w2=0.02, h2=0.05, l=2.0)),
    # HomogeneousSingleScatterer (homogeneous_single_scatterer.py:26-195)
    # with the kernels of acc/kernels
    "hss_sphere_isotropic": dict(
        kind="hss", n=256, nu=3, inputs=("along_z", 0.012, 0.012, 55.0),
        shape=("sphere", 0.01),
        kernel=dict(kind="isotropic", mu=25.0, sigma=25.0)),
    "hss_hollow_cylinder_isotropic": dict(
        kind="hss", n=256, nu=3, inputs=("along_x", 0.0125, 0.026, 60.0),
        shape=("difference", ("cylinder", 0.012, 0.05),
               ("cylinder", 0.010, 0.05)),
        kernel=dict(kind="isotropic", mu=3.0, sigma=40.0)),
    "hss_cylinder_powder": dict(
        kind="hss", n=256, nu=4, inputs=("along_x", 0.006, 0.022, 30.0),
        shape=("cylinder", 0.005, 0.04),
        kernel=dict(kind="powder", peaks=powder_peak_rows(),
                    unitcell_volume=66.4, abs=0.23, inc=0.0, coh=1.5)),
    "hss_cylinder_powder_broadened": dict(
        kind="hss", n=256, nu=4, inputs=("along_x", 0.006, 0.022, 30.0),
        shape=("cylinder", 0.005, 0.04),
        kernel=dict(kind="powder", peaks=powder_peak_rows(width=2e-3),
                    unitcell_volume=66.4, abs=0.23, inc=0.0, coh=1.5)),
    "hss_sphere_powder_al": dict(
        kind="hss", n=256, nu=4, inputs=("along_z", 0.012, 0.012, 60.0),
        shape=("sphere", 0.01),
        kernel=dict(kind="powder", peaks=AL_PEAKS,
                    unitcell_volume=AL_A ** 3, **AL_XS)),
    "hss_sphere_e_q": dict(
        kind="hss", n=256, nu=24, inputs=("along_z", 0.012, 0.012, 60.0),
        shape=("sphere", 0.01),
        kernel=dict(kind="E_Q", E_Q="30+20*sin(Q)", S_Q="1+0.1*Q",
                    Qmin=0.5, Qmax=9.0, mu=2.0, sigma=8.0)),
    "hss_sphere_constant_qe": dict(
        kind="hss", n=256, nu=4, inputs=("along_z", 0.012, 0.012, 60.0),
        shape=("sphere", 0.01),
        kernel=dict(kind="constant_qe", Q=3.0, E=30.0, mu=2.0, sigma=8.0)),
    # SNS / STS moderator sources (acc/components/sources/SNS_source.py,
    # STS_source.py) on the reference's moderator files: the arguments of
    # tests/components/sources/test_SNS_source.py:12 and
    # test_STS_source.py:28, VERDI's energy window (VERDI_base.py:32), and
    # a disc face
    "sns_source_test": dict(
        kind="sns_source", n=256, nu=6, file=SNS_FILE,
        kw=dict(Emin=5, Emax=20, xwidth=0.03, yheight=0.03, dist=5,
                focus_xw=.03, focus_yh=.03)),
    "sns_source_verdi_window": dict(
        kind="sns_source", n=256, nu=6, file=SNS_FILE,
        kw=dict(Emin=0.1, Emax=1000., xwidth=0.03, yheight=0.03, dist=6.35,
                focus_xw=0.04, focus_yh=0.04)),
    "sns_source_disc": dict(
        kind="sns_source", n=256, nu=6, file=SNS_FILE,
        kw=dict(Emin=3, Emax=60, xwidth=0, yheight=0, dist=2.0,
                focus_xw=0.02, focus_yh=0.05, radius=0.02)),
    "sts_source_test": dict(
        kind="sts_source", n=256, nu=6, file=STS_FILE,
        kw=dict(Emin=3, Emax=82, xwidth=0.03, yheight=0.03, dist=2.5,
                focus_xw=.03, focus_yh=.03)),
    # monitors (acc/components/monitors)
    "psd_monitor": dict(
        kind="psd_monitor", n=256, nu=1, inputs="plane",
        kw=dict(xwidth=0.06, yheight=0.05, nx=20, ny=24)),
    "wavelength_monitor": dict(
        kind="wavelength_monitor", n=256, nu=1, inputs="plane",
        kw=dict(xwidth=0.06, yheight=0.05, Lmin=0.5, Lmax=4.0, nchan=50)),
    "psd_monitor_4pi": dict(
        kind="psd_monitor_4pi", n=256, nu=1, inputs="isotropic",
        kw=dict(radius=3.0, nphi=30, ntheta=36)),
    "iqe_monitor": dict(
        kind="iqe_monitor", n=256, nu=1, inputs="isotropic",
        kw=dict(Ei=60.0, Qmin=0.0, Qmax=10.0, nQ=20, Emin=-45.0,
                Emax=45.0, nE=18)),
}


def draw_inputs(case, seed):
    """(n, 10) input neutrons for a case (None for a source)."""
    n = case["n"]
    rng = np.random.default_rng(seed)
    spec = case.get("inputs")
    if spec is None:
        return None
    out = np.zeros((n, 10))
    out[:, 8] = rng.uniform(0.0, 2e-3, n)
    out[:, 9] = rng.uniform(0.5, 2.0, n)
    if spec == "guide":
        # entrance plane region, +-0.6 deg divergence, 5-100 meV; a few
        # start behind or beside the opening, or fly backwards
        out[:, 0] = rng.uniform(-0.027, 0.027, n)
        out[:, 1] = rng.uniform(-0.027, 0.027, n)
        out[:, 2] = rng.uniform(-0.02, 0.0, n)
        v = SE2V * np.sqrt(rng.uniform(5.0, 100.0, n))
        ax = np.radians(rng.uniform(-0.6, 0.6, n))
        ay = np.radians(rng.uniform(-0.6, 0.6, n))
        d = np.stack([np.tan(ax), np.tan(ay), np.ones(n)], 1)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out[:, 3:6] = v[:, None] * d
        out[-4:, 5] *= -1
        return out
    if spec in ("plane", "isotropic"):
        v = SE2V * np.sqrt(rng.uniform(5.0, 100.0, n))
        if spec == "plane":
            out[:, 0] = rng.uniform(-0.04, 0.04, n)
            out[:, 1] = rng.uniform(-0.035, 0.035, n)
            out[:, 2] = rng.uniform(-0.05, 0.05, n)
            d = np.stack([rng.normal(0, 0.05, n), rng.normal(0, 0.05, n),
                          np.ones(n)], 1)
            d[-8:, 2] = -1.0
        else:
            out[:, :3] = rng.normal(0, 0.003, (n, 3))
            d = rng.normal(0, 1, (n, 3))
            d[:, 2] += 0.5
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out[:, 3:6] = v[:, None] * d
        return out
    kind, half_a, half_b, E = spec
    v = SE2V * math.sqrt(E) * rng.uniform(0.9, 1.1, n)
    a = rng.uniform(-half_a, half_a, n)
    b = rng.uniform(-half_b, half_b, n)
    if kind == "along_z":  # beam along z at z = -0.05 onto (x, y)
        out[:, 0], out[:, 1], out[:, 2] = a, b, -0.05
        d = np.stack([rng.normal(0, 0.02, n), rng.normal(0, 0.02, n),
                      np.ones(n)], 1)
    else:  # beam along x at x = -0.05 onto (y, z): across a z-axis cylinder
        out[:, 0], out[:, 1], out[:, 2] = -0.05, a, b
        d = np.stack([np.ones(n), rng.normal(0, 0.02, n),
                      rng.normal(0, 0.02, n)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out[:, 3:6] = v[:, None] * d
    return out


def draw_uniforms(case, seed):
    """(n, nu) float32 uniforms k / 2^24 (the engine's uniform grid)."""
    rng = np.random.default_rng(seed + 1000)
    k = rng.integers(0, 2 ** 24, size=(case["n"], case["nu"]))
    return (k / 2.0 ** 24).astype(np.float32)


# ------------------------------------------------------------ product side
def _product_shape(spec):
    from acc_gb300.geometry import Cylinder, Difference, Sphere
    if spec[0] == "sphere":
        return Sphere(spec[1])
    if spec[0] == "cylinder":
        return Cylinder(spec[1], spec[2])
    if spec[0] == "difference":
        return Difference(_product_shape(spec[1]), _product_shape(spec[2]))
    raise ValueError(spec)


def _product_kernel(k):
    from acc_gb300 import kernels as K
    kind = k["kind"]
    if kind == "isotropic":
        return K.IsotropicKernel(k["mu"], k["sigma"])
    if kind == "powder":
        peaks = [K.Peak(**p) for p in k["peaks"]]
        return K.SimplePowderDiffractionKernel(
            peaks, k["unitcell_volume"], absorption_cross_section=k["abs"],
            incoherent_cross_section=k["inc"],
            coherent_cross_section=k["coh"])
    if kind == "E_Q":
        return K.E_Q_Kernel(k["E_Q"], k["S_Q"], k["Qmin"], k["Qmax"],
                            k["mu"], k["sigma"])
    if kind == "constant_qe":
        return K.ConstantQEKernel(k["Q"], k["E"], k["mu"], k["sigma"])
    raise ValueError(kind)


def build_product(name):
    """The package's component for case `name`."""
    case = CASES[name]
    kind = case["kind"]
    if kind == "source":
        from acc_gb300.components.sources.source_simple import Source_simple
        return Source_simple(name, **case["kw"])
    if kind in ("sns_source", "sts_source"):
        import warnings
        from acc_gb300.components.sources.SNS_source import (SNS_source,
                                                             STS_source)
        cls = SNS_source if kind == "sns_source" else STS_source
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            return cls(name, moderator_path(case["file"]), **case["kw"])
    if kind == "guide":
        from acc_gb300.components.optics.guide import Guide
        return Guide(name, **case["kw"])
    if kind == "hss":
        from acc_gb300.components.samples.homogeneous_single_scatterer \
            import factory
        return factory(_product_shape(case["shape"]),
                       _product_kernel(case["kernel"]))(name)
    import importlib
    mod = importlib.import_module("acc_gb300.components.monitors." + kind)
    cls = {"psd_monitor": "PSD_monitor",
           "wavelength_monitor": "Wavelength_monitor",
           "psd_monitor_4pi": "PSD_monitor_4Pi",
           "iqe_monitor": "IQE_monitor"}[kind]
    return getattr(mod, cls)(name, **case["kw"])


def product_instrument(name, inputs):
    """An instrument: the case's component, fed by the stored input
    neutrons unless the component is a source."""
    import acc_gb300
    from acc_gb300.components.sources.neutronfromstorage import \
        NeutronFromStorage
    ins = acc_gb300.instrument()
    if inputs is not None:
        ins.append(NeutronFromStorage("stored", neutrons=inputs),
                   position=(0, 0, 0))
    ins.append(build_product(name), position=(0, 0, 0))
    return ins
