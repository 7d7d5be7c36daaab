"""natrix_gb300: the natrix.core per-step fluid solver on GB300 (sm_103a).

Python host over a C ABI (include/natrix.h) to hand-written CUDA kernels in
natrix_gb300/csrc, built in-tree into natrix_gb300/_lib/libnatrix_gb300.so.
"""
from .core.fluid_simulator import FluidSimulator  # noqa: F401
from .core.smooth_particles_area import SmoothParticlesArea  # noqa: F401

__version__ = "0.1.0"
