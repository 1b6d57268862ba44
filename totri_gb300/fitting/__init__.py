"""Fitting loops over the differentiable renderer (reference totri/fitting)."""
from .background import TransientBackgroundConfocal, TransientBackgroundExhaustive
from .depth_map import DepthMap, DepthMapFitting, tv_loss
from .pose import PoseFitting, Rotation, Translation, apply_transform, quaternion_apply
from .rbf import GaussianRbfBase, RbfFitting, TransientBackgroundEmpty

__all__ = ["DepthMap", "DepthMapFitting", "tv_loss", "PoseFitting", "Rotation", "Translation",
           "apply_transform", "quaternion_apply", "GaussianRbfBase", "RbfFitting",
           "TransientBackgroundEmpty", "TransientBackgroundConfocal",
           "TransientBackgroundExhaustive"]
