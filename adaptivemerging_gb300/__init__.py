"""GB300-native contact hot path of the adaptive-merging rigid-body simulator.

The CUDA kernels and the C ABI live in csrc/ (built into libam.so, declared in
include/am.h); this package holds the ctypes binding (abi.py, native.py), the
seeded scene generators (scenes.py) and the host-side mirror of the
reference's CollisionProcessor / RigidBodySystem call surface (system.py).
"""
from . import abi, scenes  # noqa: F401
