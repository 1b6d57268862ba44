"""totri_gb300.reconstruct: backprojection and f-k migration (reference totri/reconstruct)."""
from .backprojection import (BackprojectionConfocalVelten, BackprojectionExhaustiveArellano,
                             BackprojectionExhaustiveVelten, second_derivative_filter)
from .fk_migration import FkMigration, StoltInterpolation

__all__ = ["BackprojectionConfocalVelten", "BackprojectionExhaustiveArellano",
           "BackprojectionExhaustiveVelten", "second_derivative_filter", "FkMigration",
           "StoltInterpolation"]
