"""The reference demo's import path (``demo.smooth_particles_area``), served
by natrix_gb300."""
