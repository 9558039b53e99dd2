"""GB300-native collision and distance engine for RPMPLv2's RealVectorSpace path."""
from . import robots, scenes  # noqa: F401
