"""GB300-native AprilTag quad detection (drop-in for the SYCL reference's
quad-detection path).  The compute runs in libatag_gb300.so (hand-written
sm_103a CUDA); this package is the host-side mirror of the reference's
stage functions plus the batched detector."""
from . import lib, records  # noqa: F401
from .lib import AtagError, default_config, init, launch_count  # noqa: F401
