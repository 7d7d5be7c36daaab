"""``natrix.core.fluid_simulator`` import path, served by natrix_gb300."""
from natrix_gb300.core.fluid_simulator import FluidSimulator  # noqa: F401
