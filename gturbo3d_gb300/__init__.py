"""GB300-native (sm_103a) RK2 integrating-factor step of Gturbo3D.

The compute path is ``libgturbo_gb.so`` (hand-written CUDA, C-ABI in
``include/gturbo_gb.h``); this package is its Python binding and the
seeded synthetic-input generator.
"""
from .api import (Ensemble, Simulation, ForcedModes, autotune, forced_modes, forcing_amplitude,
                  forcing_increments, init_noise, make_params, memory_budget, memory_estimate, probe_alu,
                  rann, read_field, read_frame, read_params, read_seed, set_memory_budget, write_field,
                  write_frame, write_seed)

__all__ = ["Ensemble", "Simulation", "ForcedModes", "autotune", "forced_modes", "forcing_amplitude",
           "forcing_increments", "init_noise", "make_params", "memory_budget", "memory_estimate",
           "probe_alu", "rann", "set_memory_budget",
           "read_field", "read_frame", "read_params", "read_seed", "write_field", "write_frame",
           "write_seed"]
