"""Y-family gates (reference: QuantumGates/YGates.py)."""
import math
from typing import Optional

import numpy as np
import torch

from .AbstractGate import _Fixed, _Param


class YGate(_Fixed):
    _NAME, _DATA = 'Y', [[0, -1j], [1j, 0]]                    # YGates.py:15-45


class RYGate(_Param):                                          # YGates.py:48-85
    _NAME = 'RY'

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        c, s = torch.cos(self.theta / 2), torch.sin(self.theta / 2)
        return self._mat([[c, -s], [s, c]])

    @staticmethod
    def _build_np(theta):
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        return np.array([[c, -s], [s, c]], dtype=np.complex128)


class CYGate(_Fixed):                                          # YGates.py:88-121
    _NAME, _SINGLE = 'CY', False
    _DATA = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]]


class RYYGate(_Param):                                         # YGates.py:124-161
    _NAME, _SINGLE = 'RYY', False

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        c, s = torch.cos(self.theta / 2), torch.sin(self.theta / 2)
        return self._mat([[c, 0, 0, -s], [0, c, s, 0], [0, -s, c, 0], [s, 0, 0, c]])
