"""GB300-native (sm_103a) implementation of the KAPSEL-ICEP per-timestep hot path.

The product is the C-ABI shared library libicep_gb300.so (include/icep_gb300.h),
built from csrc/ by icep_kapsel_gb300.build; runtime.Simulation is its Python
handle. abi holds the ctypes mirrors of the public types.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "Simulation", "build_library"]


def build_library(force=False):
    from .build import build
    return build(force=force)


def __getattr__(name):
    if name == "Simulation":
        from .runtime import Simulation
        return Simulation
    raise AttributeError(name)
