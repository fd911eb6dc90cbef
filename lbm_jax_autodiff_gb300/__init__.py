"""GB300-native (sm_103a) D3Q19 lattice-Boltzmann hot path of jax_lbm.

The compute path is the CUDA library ``lib/liblbm_gb300.so`` (C ABI in
``include/lbm_gb300.h``); there is no CPU fallback.
"""

from . import _native
from .solver import Simulation

__all__ = ["Simulation", "_native"]
