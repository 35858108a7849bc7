"""GB300-native position-based-dynamics cloth step.

The product is libpbd_gb300.so (C ABI in include/pbd_c.h, CUDA kernels for
sm_103a in csrc/).  ``pbd`` mirrors the reference's classes over that ABI;
``scenes`` builds the synthetic cloth workloads.
"""
from .pbd import (ANCHOR, BENDING, DISTANCE, GAUSSSEIDEL, RESPONSE_MASS_WEIGHTED,  # noqa: F401
                  RESPONSE_REFERENCE, CollisionSolver, PBDError, PBDObject, SolverPBD,
                  SpatialHashSystem, load)
