"""Run an instrument script on one GPU: the drop-in for
mcvine.acc.run_script (acc/run_script.py:10-35, 291-328, 330-355).

The reference generates a Python module that inlines every component's
propagate into one Numba kernel (compile, :37-139).  Here `compile` builds
the chain description that the engine's fused kernel interprets; it also
writes it as JSON for inspection.
"""

import inspect
import json
import os
import shutil
import warnings

import numpy as np

from . import config
from .components.ComponentBase import ComponentBase
from .instrument import calcTransformations  # noqa: F401  (public API)


def _check_workdir(workdir, overwrite_datafiles):
    if os.path.exists(workdir):
        if not overwrite_datafiles:
            raise IOError(f"{workdir} already exists")
        shutil.rmtree(workdir)


def run(script, workdir, ncount, overwrite_datafiles=True, ntotalthreads=None,
        threads_per_block=None, **kwds):
    """Run the instrument defined by `script` for `ncount` neutrons and save
    every monitor into `workdir` scaled by 1/ncount (run_script.py:10-35,
    210-223).  Returns the instrument.

    Every keyword in `kwds` goes to the script's instrument factory, as in
    the reference.  The random seed and the float type come from
    acc_gb300.config (rng_seed, floattype: the reference's acc/config.py);
    the keywords `_acc_seed` and `_acc_floattype`, which no instrument
    takes, override them for one run.  An existing `workdir` raises IOError
    unless `overwrite_datafiles`."""
    from . import engine
    seed = kwds.pop("_acc_seed", None)
    floattype = kwds.pop("_acc_floattype", None)
    _check_workdir(workdir, overwrite_datafiles)
    os.makedirs(workdir)
    ncount = int(ncount)
    compiled = os.path.join(workdir, "compiled_mcvine_acc_instrument.json")
    instrument = loadInstrument(script, **kwds)
    for comp in instrument.components:
        if not isinstance(comp, ComponentBase):
            raise AssertionError(f"{comp} is not a mcvine.acc component")
    _write_description(instrument, compiled)
    for comp in instrument.components:
        if hasattr(comp, "expect_neutrons"):
            comp.expect_neutrons(ncount)
    chain = engine.chain_for_instrument(instrument)
    tpb = threads_per_block or config.threads_per_block
    st = engine.run_chain(chain, ncount, seed=seed, floattype=floattype,
                          threads_per_block=min(int(tpb), 256))
    processed = st.processed
    assert processed == ncount, (
        f"Processed neutron count {processed} does not match requested "
        f"neutron count {ncount}")
    curdir = os.path.abspath(os.curdir)
    os.chdir(workdir)
    try:
        saveMonitorOutputs(instrument, scale_factor=1.0 / ncount)
    finally:
        os.chdir(curdir)
    return instrument


def compile(script, compiled_script=None, **kwds):
    """Load the instrument and write its chain description (JSON) to
    `compiled_script`; returns that path."""
    instrument = loadInstrument(os.path.abspath(script), **kwds)
    if compiled_script is None:
        f, _ = os.path.splitext(script)
        compiled_script = f + "_compiled.json"
    _write_description(instrument, compiled_script)
    return compiled_script


def _write_description(instrument, path):
    offsets, rotmats = calcTransformations(instrument)
    desc = {
        "components": [
            {"name": getattr(c, "name", ""), "class": type(c).__name__,
             "module": type(c).__module__, "opcode": int(c.opcode),
             "propagate_params": _jsonable(getattr(c, "propagate_params", ()))}
            for c in instrument.components],
        "offsets": np.asarray(offsets).tolist(),
        "rotmats": np.asarray(rotmats).tolist(),
    }
    with open(path, "w") as f:
        json.dump(desc, f, indent=1)


def _jsonable(x):
    if isinstance(x, np.ndarray):
        return x.tolist()
    if isinstance(x, (list, tuple)):
        return [_jsonable(v) for v in x]
    if isinstance(x, (np.integer,)):
        return int(x)
    if isinstance(x, (np.floating,)):
        return float(x)
    if isinstance(x, (int, float, str, bool)) or x is None:
        return x
    return repr(x)


def saveMonitorOutputs(instrument, scale_factor=1.0):
    from .components.monitors.MonitorBase import MonitorBase
    for comp in instrument.components:
        if isinstance(comp, MonitorBase) or getattr(comp, "saves_neutrons",
                                                    False):
            comp.save(scale_factor=scale_factor)


def loadInstrument(script, **kwds):
    """Import `script`; its `instrument` is an instrument or a callable
    that makes one from the keywords it accepts (run_script.py:297-328)."""
    import importlib.util
    from . import compat
    compat.install_mcvine_alias()
    spec = importlib.util.spec_from_file_location("mcvinesim", script)
    m = importlib.util.module_from_spec(spec)
    d = os.path.dirname(os.path.abspath(script))
    import sys
    added = d not in sys.path
    if added:
        sys.path.insert(0, d)
    try:
        spec.loader.exec_module(m)
    finally:
        if added:
            sys.path.remove(d)
    assert hasattr(m, "instrument")
    instrument = m.instrument
    from .instrument import Instrument
    if not isinstance(instrument, Instrument) and not hasattr(
            instrument, "components"):
        assert callable(instrument)
        kwds = _getRelevantKwds(instrument, kwds)
        instrument = instrument(**kwds)
    return instrument


def _getRelevantKwds(method, kwds):
    """Keywords of `kwds` that `method` accepts, removed from `kwds`."""
    params = inspect.signature(method).parameters
    d = {}
    for a in list(kwds):
        if a not in params:
            warnings.warn(f"Unrecognized kwd: {a!r}")
    for a in params:
        if a in kwds:
            d[a] = kwds.pop(a)
    return d


def main(argv=None):
    """Command line: the options of run_script.py:330-355."""
    import argparse
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("script")
    ap.add_argument("--workdir", default="output")
    ap.add_argument("--ncount", type=float, default=1e6)
    ap.add_argument("--overwrite_datafiles", action="store_true")
    ap.add_argument("--total_threads", type=int, default=int(1e6))
    ap.add_argument("--threads_per_block", type=int, default=512)
    ap.add_argument("--floattype", default=None)
    ap.add_argument("--additional-kargs", default=None,
                    help="additional keyword arguments in a YAML file (JSON "
                         "where PyYAML is not installed)")
    a = ap.parse_args(argv)
    kwds = {}
    if a.additional_kargs:
        kwds = load_additional_kargs(a.additional_kargs)
    if a.floattype:
        kwds["_acc_floattype"] = a.floattype
    run(a.script, a.workdir, int(a.ncount),
        overwrite_datafiles=a.overwrite_datafiles,
        ntotalthreads=a.total_threads, threads_per_block=a.threads_per_block,
        **kwds)


def load_additional_kargs(path):
    """The keyword file of --additional-kargs: YAML, as the reference reads
    it (yaml.safe_load, run_script.py:345-346); JSON (a subset of YAML)
    when PyYAML is not installed."""
    with open(path) as f:
        text = f.read()
    try:
        import yaml
    except ImportError:
        return json.loads(text) if text.strip() else {}
    return yaml.safe_load(text) or {}


if __name__ == "__main__":
    main()
