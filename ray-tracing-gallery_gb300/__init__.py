"""GB300-native ray-tracing core: the hot path of expenses/ray-tracing-gallery
(BLAS/TLAS build and refit, traversal with a watertight triangle test,
alpha-clip any-hit, and the raygen / closest-hit / miss / shadow programs)
as sm_103a CUDA behind a C ABI (include/rtcore.h, librtcore.so).

Modules: ``abi`` (ctypes mirror of the C ABI), ``scenes`` (procedural
inputs), ``host`` (the reference's host interface over the ABI), ``build``
(nvcc build of librtcore.so).
"""
from . import abi, scenes  # noqa: F401

__all__ = ["abi", "scenes", "host", "build"]
