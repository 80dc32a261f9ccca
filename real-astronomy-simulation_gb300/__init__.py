"""GB300-native self-gravity engine: hand-written sm_103a CUDA behind a C ABI
(include/gbgrav.h), with a host-side mirror of the reference's Engine /
solver interface (Khaserdene/real-astronomy-simulation, core/engine.py,
core/solvers/gravity.py, core/solvers/barnes_hut.py).

Modules:
  engine, state, units   Engine / State drop-ins (core/engine.py, core/state.py)
  solvers.gravity        direct N^2 (core/solvers/gravity.py)
  solvers.barnes_hut     LBVH Barnes-Hut (core/solvers/barnes_hut.py)
  solvers.external       analytic galaxy potential, add_grav_ext
                         (core/living_galaxy_engine.py, core/gas_disk_engine.py)
  solvers.neighbor_grid  SPH neighbour grid (core/solvers/neighbor_grid.py)
  batch, autotune        many systems per launch, tile-shape tuning
  adjoint                gradients of the direct-sum KDK (torch.autograd)
  snapshot               snapshots written off the step loop
  ic                     seeded initial conditions (core/ic/plummer.py, disk.py)

The directory name is not a Python identifier; import it with
``importlib.import_module("real-astronomy-simulation_gb300")``.
"""
from . import units
from ._lib import GravityError, load as load_library
from .engine import Engine, init_taichi
from .state import State, PTYPE_DM, PTYPE_STAR, PTYPE_GAS

__all__ = ["Engine", "State", "GravityError", "init_taichi", "load_library", "units",
           "PTYPE_DM", "PTYPE_STAR", "PTYPE_GAS"]
