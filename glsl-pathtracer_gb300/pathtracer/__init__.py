"""GB300 path tracer: host side of the drop-in for GLSL-PathTracer's renderer.

The compute path is libptgb.so (hand-written sm_103a CUDA behind the C ABI of
include/pt_cuda.h); this package holds the ctypes bindings, the scene
container, the synthetic scene builders and a Python mirror of the
reference's Renderer interface.
"""
from . import capi  # noqa: F401
from .scene import SceneData, load_ref_dump  # noqa: F401
