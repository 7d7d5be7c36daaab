"""``demo.smooth_particles_area`` import path (demo/smooth_particles_area.py:15
of the reference), served by natrix_gb300."""
from natrix_gb300.core.smooth_particles_area import SmoothParticlesArea  # noqa: F401
