"""GB300-native distance-driven CT operators with CTLIB's API.

    import ctlib_gb300 as ctlib
    sino = ctlib.projection(image, options)      # B x 1 x V x D
    img  = ctlib.projection_t(sino, options)     # B x 1 x H x W

The operators run hand-written sm_103a CUDA kernels (``csrc/``) behind the C ABI
declared in ``include/ctgb.h``; there is no CPU path.
"""

from .ops import (backprojection, backprojection_sv, backprojection_t, clear_plans, fbp, get_plan,  # noqa: F401
                  laplacian, projection, projection_t)

__all__ = ["projection", "projection_t", "backprojection", "backprojection_t", "fbp", "backprojection_sv",
           "laplacian", "get_plan", "clear_plans"]
