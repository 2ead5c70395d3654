"""Load ``cases.py`` (or ``full_cases.py``) as a fresh module bound to one
implementation of ``xgrid``."""
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def load_cases(xgrid_module, cacheroot: str, tag: str, filename: str = "cases.py"):
    name = f"_xg{os.path.splitext(filename)[0]}_{tag}"
    spec = importlib.util.spec_from_file_location(name, os.path.join(HERE, filename))
    mod = importlib.util.module_from_spec(spec)
    mod.xgrid = xgrid_module
    mod.CACHEROOT = cacheroot
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod
