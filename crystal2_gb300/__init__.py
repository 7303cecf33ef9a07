"""GB300 (sm_103a) path-tracing hot path for the Crystal2 renderer.

The compute path is ``libc2g.so`` (C++ host library + hand-written CUDA kernels) behind the C ABI
of ``include/c2g.h``; this package is its Python binding, the reference-shaped driver
(``RayTracer``, ``Integrator``) and the seeded scene generators used by the tests and the bench.
"""
from ._native import C2GError, load_library  # noqa: F401
from . import _native as native  # noqa: F401
from .renderer import Batch, Context, Integrator, RayTracer, write_hdr  # noqa: F401

__all__ = ["C2GError", "Context", "Integrator", "RayTracer", "load_library", "native", "write_hdr"]
