"""GB300-native self-gravity engine: hand-written sm_103a CUDA behind a C ABI
(include/gbgrav.h), with a host-side mirror of the reference's Engine /
solver interface (Khaserdene/real-astronomy-simulation, core/engine.py,
core/solvers/gravity.py, core/solvers/barnes_hut.py).

The directory name is not a Python identifier; import it with
``importlib.import_module("real-astronomy-simulation_gb300")``.
"""
from . import units
from ._lib import GravityError, load as load_library
from .engine import Engine, init_taichi
from .state import State, PTYPE_DM, PTYPE_STAR, PTYPE_GAS

__all__ = ["Engine", "State", "GravityError", "init_taichi", "load_library", "units",
           "PTYPE_DM", "PTYPE_STAR", "PTYPE_GAS"]
