"""The demo's ``SmoothParticlesArea`` under the natrix.core import path."""
from natrix_gb300.core.smooth_particles_area import SmoothParticlesArea  # noqa: F401
