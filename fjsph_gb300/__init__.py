"""GB300-native WCSPH hot path of FJSPH: neighbour search, residual and integrators as sm_103a
kernels behind a C ABI (include/fjsph_gb300.h), with a Python host mirror of the reference's
function interface."""
from . import _cdefs as cdefs
from .state import SPHState, BlockSpec, InletSpec

__all__ = ["cdefs", "SPHState", "BlockSpec", "InletSpec", "Context"]


def __getattr__(name):
    if name == "Context":
        from .api import Context
        return Context
    raise AttributeError(name)
