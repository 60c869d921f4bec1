"""newrecon_gb300 -- GB300-native OSTR reconstruction for digital breast tomosynthesis."""
from .geometry import Geometry, config, view_angles  # noqa: F401

__version__ = "0.1.0"
