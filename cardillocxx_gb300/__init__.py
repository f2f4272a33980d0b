"""cardillocxx_gb300 -- GB300-native contact hot path of CardilloCxx.

The Moreau midpoint step for sphere scenes (uniform-grid broad phase, sphere-sphere /
sphere-halfspace / sphere-drum narrow phase, projected Jacobi over Coulomb disk cones applied
matrix-free as G M^-1 G^T, velocity and quaternion update) as hand-written sm_103a CUDA kernels
behind the C ABI in include/cdx.h. This package is the Python view of that library: it loads
libcdx.so (built in-tree by build.py) and fails loudly when it is missing.
"""
from ._lib import CdxError, lib  # noqa: F401
from .engine import Config, PhysicsEngine  # noqa: F401
from . import scenes  # noqa: F401
