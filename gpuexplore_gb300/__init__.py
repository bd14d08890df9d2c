"""gpuexplore_gb300: GB300-native on-the-fly state-space exploration of gpf networks.

The product is ``_lib/libgpx.so`` (CUDA kernels for sm_103a behind the C ABI in
``include/gpx.h``) and the ``_lib/gpuexplore`` command-line tool.  This package
holds the ctypes binding (:mod:`.lib`), the gpf format (:mod:`.gpf`), the seeded
network generators (:mod:`.gen`) and the in-tree build (:mod:`.build`).
"""
from . import gpf, gen  # noqa: F401

__all__ = ["gpf", "gen"]
