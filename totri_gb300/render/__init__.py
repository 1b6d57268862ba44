"""totri_gb300.render: differentiable transient renderers (reference totri/render)."""
from .mesh import MeshRenderConfocal, MeshRenderExhaustive

__all__ = ["MeshRenderConfocal", "MeshRenderExhaustive"]
