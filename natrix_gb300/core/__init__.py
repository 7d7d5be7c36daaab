"""Drop-in counterparts of natrix.core's simulator classes."""
