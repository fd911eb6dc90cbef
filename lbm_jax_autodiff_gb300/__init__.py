"""GB300-native (sm_103a) D3Q19 lattice-Boltzmann hot path of jax_lbm.

The compute path is the CUDA library ``lib/liblbm_gb300.so`` (C ABI in
``include/lbm_gb300.h``); there is no CPU fallback.  The public names follow
``jax_lbm`` so that drivers written against it run unchanged on torch CUDA
tensors.
"""

from . import _native
from .core.boundary import zou_he_inlet, zou_he_outlet
from .core.collision import bgk, mrt, smagorinsky_tau
from .core.equilibrium import compute_density, compute_velocity, equilibrium
from .core.forces import drag_coefficient, momentum_exchange, projected_area
from .core.lattice import CS2, D3Q19_OPPOSITE, D3Q19_VELOCITIES, D3Q19_WEIGHTS
from .core.streaming import stream
from .batch import Batch
from .solver import Simulation
from .state import LBMParams, LBMState, clear_handles, simulate, step

__all__ = [
    "D3Q19_VELOCITIES", "D3Q19_WEIGHTS", "D3Q19_OPPOSITE", "CS2",
    "equilibrium", "compute_density", "compute_velocity",
    "bgk", "mrt", "smagorinsky_tau", "stream", "zou_he_inlet", "zou_he_outlet",
    "momentum_exchange", "drag_coefficient", "projected_area",
    "LBMState", "LBMParams", "step", "simulate", "clear_handles", "Simulation", "Batch",
]
