"""Import alias so code written against the reference package
(``from natrix.core.fluid_simulator import FluidSimulator``) runs on
natrix_gb300 unchanged."""
from natrix_gb300 import FluidSimulator, SmoothParticlesArea  # noqa: F401
