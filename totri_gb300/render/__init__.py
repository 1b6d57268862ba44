"""totri_gb300.render: differentiable transient renderers (reference totri/render)."""
from .mesh import MeshRenderConfocal, MeshRenderExhaustive
from .volume import VolumeRenderConfocal, VolumeRenderExhaustive

__all__ = ["MeshRenderConfocal", "MeshRenderExhaustive", "VolumeRenderConfocal",
           "VolumeRenderExhaustive"]
