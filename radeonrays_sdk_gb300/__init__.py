"""GB300-native RadeonRays BVH build + ray intersection.

The product is librr.so (C-ABI, include/radeonrays.h + include/radeonrays_cuda.h)
built from csrc/ for sm_103a.  This package holds its build script, a ctypes
binding (rr), seeded synthetic workloads (scenes) and the serving loop
(serving).
"""
from . import rr, scenes  # noqa: F401

__all__ = ["rr", "scenes"]
