"""GB300-native collision and distance engine for RPMPLv2's RealVectorSpace path."""
import os

# Up to 32 hardware work queues instead of CUDA's default 8, so the serving
# loop's express and bulk streams (and a caller's own streams) do not share a
# queue, which would order their work behind one another.  It takes effect
# only when set before the process creates its CUDA context; a value already
# in the environment is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import robots, scenes  # noqa: F401,E402
