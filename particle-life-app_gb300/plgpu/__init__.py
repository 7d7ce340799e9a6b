"""plgpu — GB300-native Particle Life physics step behind the reference's API.

The compute path is the CUDA library libplgpu.so (C ABI, include/plgpu.h);
this package builds it, binds it with ctypes and mirrors the reference's
Physics / PhysicsSettings / Matrix / Accelerator surface on top of it.
"""
from . import _build, _lib
from ._lib import PlgError, load
from .physics import (
    DefaultMatrix,
    DefaultMatrixGenerator,
    DefaultPositionSetter,
    DefaultTypeSetter,
    GpuWorld,
    ParticleLifeAccelerator,
    Physics,
    PhysicsSettings,
)

__all__ = [
    "DefaultMatrix",
    "DefaultMatrixGenerator",
    "DefaultPositionSetter",
    "DefaultTypeSetter",
    "GpuWorld",
    "ParticleLifeAccelerator",
    "Physics",
    "PhysicsSettings",
    "PlgError",
    "load",
    "_build",
    "_lib",
]
