"""totri_gb300.reconstruct: backprojection (reference totri/reconstruct)."""
