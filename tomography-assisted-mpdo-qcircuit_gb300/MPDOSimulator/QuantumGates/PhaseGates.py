"""Phase gates (reference: QuantumGates/PhaseGates.py)."""
import math
from typing import Optional

import torch

from .AbstractGate import _Fixed, _Param, _cexp


class SGate(_Fixed):
    _NAME, _DATA = 'S', [[1, 0], [0, 1j]]                      # PhaseGates.py:16-46


class SDGGate(_Fixed):
    _NAME, _DATA = 'Sdg', [[1, 0], [0, -1j]]                   # PhaseGates.py:49-79


class TGate(_Fixed):
    _NAME, _DATA = 'T', [[1, 0], [0, (1 + 1j) / math.sqrt(2)]]  # PhaseGates.py:82-112


class PGate(_Param):                                           # PhaseGates.py:115-151
    _NAME = 'P'

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        return self._mat([[1, 0], [0, _cexp(self.theta)]])


class CPGate(_Param):                                          # PhaseGates.py:154-190
    _NAME, _SINGLE = 'CP', False

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        return self._mat([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, _cexp(self.theta)]])
