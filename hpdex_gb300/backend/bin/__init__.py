"""Native extension namespace, mirroring the reference's hpdex.backend.bin package."""
from . import kernel  # noqa: F401
