"""GB300-native drop-in for the nBounce path-tracing compute pass.

The compute path is ``libnbounce.so`` (hand-written sm_103a CUDA kernels behind the C ABI
in ``include/nbounce.h``); this package only binds it and supplies seeded workloads.
"""
from ._lib import NbError, lib  # noqa: F401
from .cache import RadianceCache  # noqa: F401
from .pathtracer import (EnvMap, Globals, Pathtracer, SceneBuffers, bvh_build, camera_struct,  # noqa: F401
                         sobol_burley_table)
