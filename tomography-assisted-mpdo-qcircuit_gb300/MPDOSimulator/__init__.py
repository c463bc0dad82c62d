"""GB300-native drop-in for the reference's ``MPDOSimulator`` package.

Same import surface (``TensorCircuit``, ``Tools``, ``dmOperations``); the
MPDO evolution and readout run on the GPU through ``mpdo_gb300``.
"""
__version__ = '1.0.0'

from . import Tools  # noqa: F401
from . import dmOperations  # noqa: F401
from .Circuit import TensorCircuit, evolve_batch  # noqa: F401

__all__ = ['TensorCircuit', 'Tools', 'dmOperations', 'evolve_batch']
