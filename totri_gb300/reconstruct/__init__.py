"""totri_gb300.reconstruct: backprojection (reference totri/reconstruct)."""
from .backprojection import (BackprojectionConfocalVelten, BackprojectionExhaustiveArellano,
                             BackprojectionExhaustiveVelten, second_derivative_filter)

__all__ = ["BackprojectionConfocalVelten", "BackprojectionExhaustiveArellano",
           "BackprojectionExhaustiveVelten", "second_derivative_filter"]
