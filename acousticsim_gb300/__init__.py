"""GB300 (sm_103a) implementation of AcousticSim's Baraff-Witkin implicit cloth step.

The compute path is libcloth_gb300.so (hand-written CUDA + C ABI, see
include/cloth_gb300.h); this package holds the ctypes bindings and the
Python mirror of the reference's cloth API.
"""
from . import _native
from ._native import ClothError, REFERENCE_PARAMS, SolveParams, params
from .cloth import (BaraffClothGpu, ClothBody, ClothContext, ClothServer, build_grid,
                    kinematic_pose, load_obj_mesh)

__all__ = ["BaraffClothGpu", "ClothBody", "ClothContext", "ClothError", "ClothServer", "REFERENCE_PARAMS", "SolveParams",
           "build_grid", "kinematic_pose", "load_obj_mesh", "params", "load_library"]


def load_library():
    """Load libcloth_gb300.so; raises ImportError when it has not been built."""
    return _native.load()
