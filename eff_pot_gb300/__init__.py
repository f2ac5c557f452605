"""eff_pot_gb300: GB300-native Orsay-Trento helium order-parameter evolution.

The package is the host side of libeffpot.so (CUDA, sm_103a): the C ABI in
include/eff_pot.h does all the work on the GPU; this package binds it with
ctypes and mirrors the reference's subroutine interface (Solver).
"""
from . import _abi
from .config import (make_config, config_dict, morse, koutselos, null_potential, patil, aziz_he, tang_toennies,
                     series_potential, DEFAULTS, KTOPS, MP_U)
from .solver import (Solver, Batch, EffPotError, load_library, library_config_defaults, select_pot,
                     potential_values, LIBPATH)
from .initial import woods_saxon_psi, grid_axes

__all__ = [
    "Solver", "Batch", "EffPotError", "load_library", "library_config_defaults", "make_config",
    "config_dict", "morse", "koutselos", "null_potential", "patil", "aziz_he", "tang_toennies",
    "series_potential", "select_pot", "potential_values", "woods_saxon_psi", "grid_axes", "DEFAULTS",
    "KTOPS", "MP_U", "LIBPATH",
]
