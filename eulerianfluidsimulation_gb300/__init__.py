"""GB300 (sm_103a) Eulerian liquid step: Stable-Fluids advection and projection with Chentanez-Mueller
mass-conserving density correction, behind the reference simulator-backend interface.

The compute path is ``libefs_gb300.so`` (hand-written CUDA kernels behind the C ABI of
``include/efs_gb300.h``); this package is its host-side binding.
"""
from . import abi
from .abi import EfsParams, EfsStats, params_default
from ._lib import EfsError, LIB_PATH
from .simulator import (GB300Batch2D, GB300Simulator2D, GB300Simulator3D, device_count, params_dam, scene_batch2d,
                        scene_dam2d, scene_dam3d, unet_param_count)

__all__ = ["abi", "EfsParams", "EfsStats", "EfsError", "LIB_PATH", "GB300Batch2D", "GB300Simulator2D",
           "GB300Simulator3D", "device_count", "params_dam", "params_default", "scene_batch2d", "scene_dam2d",
           "scene_dam3d", "unet_param_count"]
