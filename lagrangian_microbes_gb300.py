"""Import name of the package stored in the directory ``lagrangian-microbes_gb300/``.

A directory name with a hyphen cannot be imported directly, so this module loads that directory
as the package ``lagrangian_microbes_gb300`` and replaces itself in ``sys.modules``:
``import lagrangian_microbes_gb300`` then behaves like a normal package import.
"""

import importlib.util
import os
import sys

_PKG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lagrangian-microbes_gb300")
_spec = importlib.util.spec_from_file_location(
    __name__, os.path.join(_PKG_DIR, "__init__.py"), submodule_search_locations=[_PKG_DIR]
)
_module = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _module
_spec.loader.exec_module(_module)
