"""GB300-native MHFEM time-step library: Python host mirror of the C ABI.

The package directory is ``tnl-mhfem_gb300/``; add it to ``sys.path`` and
``import mhfem``.
"""
from ._lib import MhfemError, load  # noqa: F401
from .solver import Solver, StaticConfig  # noqa: F401
