"""GB300 (sm_103a) QG-YBJ+ time step behind the reference's routine interfaces.

The compute path is libqgybj.so (CUDA, built in-tree); this package is the
host side: the ctypes binding of the C-ABI, run configurations with the
seeded initial-condition generator, and the Simulation host class.
"""
from ._lib import LIB_PATH, QgError, lib  # noqa: F401
from .config import CONFIGS, RunConfig, ensemble_members, make_initial_condition, model_parameters  # noqa: F401
from .model import Ensemble, Simulation, autotune, make_config, simulation_for  # noqa: F401
