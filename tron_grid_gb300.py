"""Import shim: `import tron_grid_gb300` loads the package in ./tron-grid_gb300/.

The package directory's name contains a hyphen, which a Python import statement
cannot spell; this module registers it under the importable name.
"""
import importlib.util as _u
import os as _os
import sys as _sys

_dir = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "tron-grid_gb300")
_spec = _u.spec_from_file_location(__name__, _os.path.join(_dir, "__init__.py"), submodule_search_locations=[_dir])
_mod = _u.module_from_spec(_spec)
_sys.modules[__name__] = _mod
_spec.loader.exec_module(_mod)
