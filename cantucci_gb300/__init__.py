"""GB300 (sm_103a) Mandelbulb distance estimation, span meshing and sphere
tracing behind cantucci's Shape / MeshBuffer API.

The compute lives in libcantucci_gpu.so (include/cantucci_gpu.h); this
package is the host-side mirror of the reference's Rust interface.
Submodules: lod (ShapeMesh level of detail), batch (many spans in one run),
autograd (adjoint and forward-mode gradients), fit (depth maps and fitting).
"""
from ._ffi import CantucciError, VERTEX_DTYPE, load  # noqa: F401
from .api import (Mandelbulb, MandelbulbPolar, MeshBuffer, Mesher, Shape, Span, Sphere,  # noqa: F401
                  Timings, create_spans, march)

__version__ = "0.1.0"
