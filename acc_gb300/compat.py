"""Let instrument scripts written for mcvine.acc import this package.

`install_mcvine_alias()` makes `import mcvine` give a small module with
`instrument()` and makes every `mcvine.acc.X` import resolve to
`acc_gb300.X` (same module paths and class names as the reference, e.g.
mcvine.acc.components.sources.source_simple.Source_simple).  It does nothing
when a real mcvine installation is importable, unless force=True.
"""

import importlib
import importlib.abc
import importlib.machinery
import importlib.util
import sys
import types

_PREFIX = "mcvine.acc"


class _AliasLoader(importlib.abc.Loader):
    def __init__(self, target):
        self.target = target

    def create_module(self, spec):
        return importlib.import_module(self.target)

    def exec_module(self, module):
        pass


class _AliasFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        if fullname == _PREFIX or fullname.startswith(_PREFIX + "."):
            real = "acc_gb300" + fullname[len(_PREFIX):]
            if importlib.util.find_spec(real) is None:
                return None
            return importlib.machinery.ModuleSpec(
                fullname, _AliasLoader(real), is_package=True)
        return None


_installed = False


def install_mcvine_alias(force=False):
    global _installed
    if _installed:
        return True
    if not force:
        existing = sys.modules.get("mcvine")
        if existing is None:
            try:
                spec = importlib.util.find_spec("mcvine")
            except (ImportError, ValueError):
                spec = None
            if spec is not None:
                return False
        elif not getattr(existing, "_acc_gb300_alias", False):
            return False
    from .instrument import instrument as make_instrument
    m = types.ModuleType("mcvine")
    m.__path__ = []
    m._acc_gb300_alias = True
    m.instrument = make_instrument
    sys.modules["mcvine"] = m
    sys.meta_path.insert(0, _AliasFinder())
    _installed = True
    return True
