"""GB300-native Brinkman-Stokes flow-topology-optimization hot path.

The product is the C ABI library ``libstokes_gb300.so`` (include/stokes_gb300.h) and the
``fluid_topo`` driver; :mod:`stokes_to_gb300.capi` is its ctypes binding.
"""
from . import capi  # noqa: F401

__all__ = ["capi"]
