"""woo_gb300 -- a GB300-native DEM timestep with Woo's engine/functor surface.

One GPU engine (GpuDemEngine) replaces Woo's Leapfrog + InsertionSortCollider + ContactLoop trio.
The compute path is libwdem.so (hand-written sm_103a CUDA kernels behind the C ABI of
include/wdem.h); there is no CPU fallback.
"""
__version__ = "0.1.0"

from . import abi, core, dem, models, pack, scenes, utils  # noqa: E402,F401
from .core import Scene  # noqa: E402,F401
from .dem import master  # noqa: E402,F401
from .dem import (DemField, FrictMat, HertzMat, Sphere, Wall, Ellipsoid, Capsule, Facet, GpuDemEngine,  # noqa: E402,F401
                  Leapfrog, InsertionSortCollider, ContactLoop)
