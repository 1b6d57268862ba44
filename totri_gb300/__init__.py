"""totri_gb300: GB300-native (sm_103a) transient rendering for NLOS imaging.

A drop-in for totrilib's differentiable transient-rendering path: the mesh and
volume renderers (``totri_gb300.render``), backprojection
(``totri_gb300.reconstruct``), RBF-to-volume splatting (``totri_gb300.util``)
and the reference's native module (``totri_gb300.totri_cpp``), all backed by
hand-written CUDA kernels in libtotri_gb300.so behind a C ABI
(include/totri_gb300.h).
"""
from . import data, types
from .types import C0, BinDef, VolumeDef

__version__ = "0.1.0"

__all__ = ["BinDef", "VolumeDef", "C0", "data", "types"]
