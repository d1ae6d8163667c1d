"""gravis_gb300: GB300 (sm_103a) engine for the hot path of gravis sim-core.

The compute lives in libgvs.so (CUDA C++, C ABI in include/gvs.h).  This
package mirrors sim-core's interfaces on top of that ABI (see engine.py).
"""
from ._lib import (ALGO_BH, ALGO_DIRECT, ALGO_NONE, PREC_FP32, PREC_FP64, PREC_FP64_EXACT, PREC_MIXED, GvsError,
                   load)
from .engine import (BarnesHut, BruteForce, ColdCollapse, Context, Diagnostics, EvrardCollapse, GravitySolver,
                     LeapfrogKDK,
                     NoGravity, Particles, PlummerSphere, Snapshot, SphSolver, TwoBody, collision, compute_diagnostics,
                     default_context, ensemble_sizes, gas_sphere_1r, step_with_sph)

__all__ = ["ALGO_BH", "ALGO_DIRECT", "ALGO_NONE", "PREC_FP32", "PREC_FP64", "PREC_FP64_EXACT", "PREC_MIXED",
           "GvsError", "load", "BarnesHut", "BruteForce", "ColdCollapse", "Context", "Diagnostics", "EvrardCollapse",
           "GravitySolver", "LeapfrogKDK", "NoGravity", "Particles", "PlummerSphere", "Snapshot", "SphSolver", "TwoBody", "collision",
           "compute_diagnostics", "default_context", "ensemble_sizes", "gas_sphere_1r", "step_with_sph"]
