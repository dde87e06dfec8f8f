"""GB300-native full-state gate engine with the API of
TysonRayJones/Distributed-Full-State-Algorithms.

The compute path is ``libdfs_gb300.so`` (hand-written sm_103a kernels behind
the C ABI in ``include/dfs_gb300.h``); this package is its Python front-end.
The directory name is not an importable identifier, so ``__graft_entry__.package()``
(or ``importlib`` with ``submodule_search_locations``) loads it as ``dfs_gb300``.
"""
from .api import *  # noqa: F401,F403
from .api import __all__ as _api_all
from ._lib import C128, C128_NATIVE, C64, DfsError, load as load_library
from .circuit import Batch, Circuit, expectation
from . import state_file

__all__ = list(_api_all) + ["C128", "C128_NATIVE", "C64", "load_library", "Circuit", "Batch", "expectation",
                            "state_file"]
