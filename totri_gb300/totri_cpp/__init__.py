"""Drop-in replacement of the reference's native module ``totri_cpp``.

``from totri_gb300.totri_cpp.render import mesh_confocal_forward`` gives the
same callable (name, argument order, layouts, in-place semantics) as
``from totri_cpp.render import mesh_confocal_forward`` in the reference
(src/totri.cpp:13-54), backed by libtotri_gb300.so.
"""
from . import reconstruct, render, util

__version__ = "0.1.0"

__all__ = ["render", "reconstruct", "util"]
