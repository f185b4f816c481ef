"""GB300-native SCFT hot path (pseudo-spectral propagators, densities, field update).

Import this package by its directory name with importlib (the name contains a
hyphen): ``importlib.import_module("stimuli-responsive-nanodroplets_gb300")``.
"""
from .surface import FIELDS, Surface, chi_macro  # noqa: F401
from .solver import (SPECIES, Derived, IterOut, Solver, derive, noise_fill, read_counter,  # noqa: F401
                     read_mask, read_restart_fields, read_restart_random, set_file_names, write_energies,
                     write_run_params, write_snapshot, write_volume_error)
from . import configs  # noqa: F401
