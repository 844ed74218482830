"""brass-pan on GB300: the unified position-based particle solver step as
hand-written sm_103a CUDA behind a C ABI (include/brasspan.h).

The directory name is not a Python identifier; `load_package()` in
__graft_entry__.py registers it as the module `brasspan_gb300`.
"""
from . import abi, scenes
from .abi import BrassPanError
from .scenes import Scene
from .solver import BatchSolver, ParticleSolver, make_params

__all__ = ["abi", "scenes", "Scene", "ParticleSolver", "BatchSolver", "make_params", "BrassPanError"]
