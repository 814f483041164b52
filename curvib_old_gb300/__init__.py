"""GB300 implementation of CURVIB's pressure-projection path (PoissonRHS,
PoissonLHSNew, PoissonSolver_MG, VolumeFlux_rev, UpdatePressure, Projection)
behind the C ABI of include/cvb.h.  The compute runs in libcvb.so (CUDA for
sm_103a); this package holds its Python front-end and the synthetic-workload
generator."""
from . import workload  # noqa: F401

__all__ = ["workload", "solver", "build"]
