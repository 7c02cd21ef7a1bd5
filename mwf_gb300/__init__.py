"""GB300-native (sm_103a) timestep of Model Waleffe Flow: dealiased transforms, Galerkin
mode coupling and the AB2 / implicit update, behind a C ABI (include/mwf_gpu.h)."""
from .solver import RunParams, Ensemble, Velocity, footprint_bytes, describe_run, dof_steps, round_23, is_23_smooth
from ._lib import MwfError
from . import ic, state_io

__all__ = ["RunParams", "Ensemble", "Velocity", "footprint_bytes", "describe_run", "dof_steps", "round_23",
           "is_23_smooth", "MwfError", "ic", "state_io"]
