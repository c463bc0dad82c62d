"""GB300-native MPDO engine: C-ABI library + Python handles.

``build()`` compiles the CUDA library in-tree; ``Engine``/``Chain`` drive it.
"""
import os as _os

# The batch runner drives one stream per worker engine; the default of 8
# hardware work queues would make streams beyond the eighth share queues and
# serialise.  Takes effect only if no CUDA context exists yet in the process.
_os.environ.setdefault('CUDA_DEVICE_MAX_CONNECTIONS', '32')

from ._build import build, LIB  # noqa: E402,F401
from .engine import Engine, Chain, Batch  # noqa: E402,F401
