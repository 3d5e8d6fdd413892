"""GB300-native PIC cycle: Yee field solver, Boris push with form-factor gather,
Esirkepov deposition and supercell bookkeeping, hand-written CUDA for sm_103a
behind the C-ABI of include/picgb.h (libpicgb.so, built in-tree)."""
from . import _lib, adjoint
from ._lib import PicError, load
from .adjoint import DiffPIC, DiffSpecies
from .ensemble import Ensemble, autotune, plasma_init
from .simulation import DataConnector, Grid, Simulation, Species
from .start import quiet_start

__all__ = ["DataConnector", "DiffPIC", "DiffSpecies", "Ensemble", "Grid", "PicError", "Simulation", "Species", "autotune", "load", "plasma_init",
           "quiet_start", "adjoint", "_lib"]
