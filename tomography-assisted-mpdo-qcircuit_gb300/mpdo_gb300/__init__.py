"""GB300-native MPDO engine: C-ABI library + Python handles.

``build()`` compiles the CUDA library in-tree; ``Engine``/``Chain`` drive it.
"""
from ._build import build, LIB  # noqa: F401
from .engine import Engine, Chain  # noqa: F401
