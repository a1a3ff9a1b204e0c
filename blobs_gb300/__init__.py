"""GB300-native (sm_103a) implementation of the blobs per-step simulation path.

The product is libblobs_gb300.so (CUDA kernels + the C ABI of
include/blobs_gpu.h).  `native.World` is its Python binding; `scenes` builds
seeded synthetic worlds.
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "native"]
