"""X-family gates (reference: QuantumGates/XGates.py)."""
import math
from typing import Optional

import numpy as np
import torch

from .AbstractGate import _Fixed, _Param


class XGate(_Fixed):
    _NAME, _DATA = 'X', [[0, 1], [1, 0]]                       # XGates.py:15-45


class RXGate(_Param):                                          # XGates.py:48-85
    _NAME = 'RX'

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        c, s = torch.cos(self.theta / 2), torch.sin(self.theta / 2)
        return self._mat([[c, -1j * s], [-1j * s, c]])

    @staticmethod
    def _build_np(theta):
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)


class CXGate(_Fixed):                                          # XGates.py:88-120
    _NAME, _SINGLE = 'CX', False
    _DATA = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]


class RXXGate(_Param):                                         # XGates.py:123-160
    _NAME, _SINGLE = 'RXX', False

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        c, s = torch.cos(self.theta / 2), -1j * torch.sin(self.theta / 2)
        return self._mat([[c, 0, 0, s], [0, c, s, 0], [0, s, c, 0], [s, 0, 0, c]])
