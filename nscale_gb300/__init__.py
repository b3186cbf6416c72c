"""nscale_gb300 — GB300-native (sm_103a) nuclei-segmentation hot path of nscale."""

import os as _os

# The batched form keeps up to 32 tiles in flight, one CUDA stream each.  With
# the default 8 hardware work queues, streams share queues and a tile's short
# kernels wait behind another tile's long ones; 32 queues (the maximum) remove
# that false serialisation (measured on GB300: 530 -> 657 Mpixel/s at 16
# tiles in flight).  Read when the CUDA context is created, so it only takes
# effect when this package is imported before the first CUDA call; a value
# the caller has set is kept.
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
