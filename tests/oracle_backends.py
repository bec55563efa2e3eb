"""Oracle-backed stand-ins for the GPU propagation backends (tests only)."""
from oracle.shooting import OracleShootingBackend  # noqa: F401
