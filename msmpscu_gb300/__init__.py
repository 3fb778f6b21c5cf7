"""GB300-native many-body (FS / EAM) MD hot path of msmpscu: device neighbour list, force
passes and velocity Verlet behind a C ABI (include/msmgb.h, libmsmgb.so)."""
from . import _lib
from .engine import Engine, ForceTable, MSMError
from . import lattice

__all__ = ["Engine", "ForceTable", "MSMError", "lattice", "_lib"]
