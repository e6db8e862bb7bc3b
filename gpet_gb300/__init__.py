"""gpet_gb300 - GB300-native gPET hot path.

The simulation itself is libgpet.so (C ABI in include/gpet.h: C++ host runtime
plus hand-written sm_103a CUDA kernels). This package holds its sources
(csrc/), the build recipe (build.py), a ctypes mirror of the C ABI (api.py),
readers/writers for gPET's file formats (formats.py) and generators of seeded
synthetic workloads in those formats (scenes.py).
"""
from . import formats, scenes  # noqa: F401
from .api import Context, GpetError, load_library  # noqa: F401
