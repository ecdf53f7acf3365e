"""filament_gb: host side of the GB300 per-z-step propagation loop.

Mirrors Filament.jl's user API (src/Filament.jl:48-108): `prepare(deck)`
then `run(input)`.  All per-step work runs in libfilament_gb.so (CUDA,
sm_103a) through the C ABI of include/filament_gb.h.
"""
from .input import prepare
from .filament import run, Simulation, main_loop
from .backend import load_library, library_path, Handle, Batch
from . import _abi

from . import sweep

__all__ = ["prepare", "run", "Simulation", "main_loop", "load_library",
           "library_path", "Handle", "Batch", "sweep"]
