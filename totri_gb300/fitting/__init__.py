"""Fitting loops over the differentiable renderer (reference totri/fitting)."""
from .pose import PoseFitting, Rotation, Translation, apply_transform, quaternion_apply

__all__ = ["PoseFitting", "Rotation", "Translation", "apply_transform", "quaternion_apply"]
