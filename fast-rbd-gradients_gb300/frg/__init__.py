"""fast-rbd-gradients for GB300: the iiwa_14 forward-dynamics gradient on sm_103a.

The engine is the C ABI of include/frg.h (libfrg.so, CUDA only); this package
builds it (frg.build) and binds it (frg.native).  Importing the package does
not load the library; the first engine call does, and raises FrgError if the
library is missing.
"""
from .inputs import JOINT_LIMITS, NUM_JOINTS, perturb, ragged_horizons, sample_knots  # noqa: F401
from .native import (  # noqa: F401
    DQDD_FLOATS,
    KNOT_NONFINITE_INPUT,
    KNOT_NONFINITE_OUTPUT,
    MINV_FLOATS,
    Context,
    FrgError,
    Plan,
    Server,
    dims,
    forward_dynamics_gradient,
    lib,
    model_name,
)
