"""Samples (acc/components/samples): the sample-assembly helpers of
acc/components/samples/__init__.py:1-48.

    hs = loadFirstHomogeneousScatterer(path_to_sampleassembly_xml)
    HSSbase = factory(shape=hs.shape(), kernel=hs.kernel())

The assembly files are read by acc_gb300.sampleassembly (the subset of
mcvine's sampleassembly / mccomponents formats the reference's sample
scripts use).
"""


def loadScattererComposite(sampleassembly_xml):
    """The scatterers of a sample assembly file (:4-23)."""
    from acc_gb300.sampleassembly import load
    return load(sampleassembly_xml)


def loadFirstHomogeneousScatterer(sampleassembly_xml):
    """The first scatterer of a sample assembly file (:25-27): an object
    with shape() and kernel()."""
    return loadScattererComposite(sampleassembly_xml).elements()[0]


def getAbsScttCoeffs(kernel):
    """(absorption coefficient at 2200 m/s, scattering coefficient) of a
    kernel, 1/m (:29-48): its own absorption_coefficient and
    scattering_coefficient (a powder kernel's scattering depends on the
    neutron's speed and is None here)."""
    mu = getattr(kernel, "absorption_coefficient", None)
    sigma = getattr(kernel, "scattering_coefficient", None)
    if mu is None:
        raise ValueError(f"{kernel!r} has no absorption coefficient")
    return float(mu), (None if sigma is None else float(sigma))
