"""GB300-native engine for OpFlow's explicit-evaluation and implicit-solve paths.

The compute lives in libopflow_gpu.so (hand-written sm_103a kernels behind the C ABI declared in
include/opflow_gpu.h); this package is the Python mirror of OpFlow's API on top of it.
"""
from ._capi import OpflowError, launch_count  # noqa: F401
from .api import (  # noqa: F401
    BCType, CartesianField, Eq, CartesianMesh, Context, DimPos, Equation, Expr, ExprBuilder, LocOnMesh, MeshBuilder,
    d1, d1IntpCenterToCorner, d1_weno53_downwind, d1_weno53_upwind, d2, d2x, d2y, d2z, default_context, describe, dx,
    dy, dz, serialize, StructSolverParams, EqnSolveState, EqnSolveHandler, makeEqnSolveHandler, Solve, assemble, weno_rk3, Problem, Batch, Server,
)

__version__ = "0.1.0"
