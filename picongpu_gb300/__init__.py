"""GB300-native PIC cycle: Yee field solver, Boris push with form-factor gather,
Esirkepov deposition and supercell bookkeeping, hand-written CUDA for sm_103a
behind the C-ABI of include/picgb.h (libpicgb.so, built in-tree)."""
from . import _lib
from ._lib import PicError, load
from .ensemble import Ensemble, autotune, plasma_init
from .simulation import DataConnector, Grid, Simulation, Species

__all__ = ["DataConnector", "Ensemble", "Grid", "PicError", "Simulation", "Species", "autotune", "load", "plasma_init",
           "_lib"]
