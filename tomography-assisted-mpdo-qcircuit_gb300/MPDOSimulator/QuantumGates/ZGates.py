"""Z-family gates (reference: QuantumGates/ZGates.py)."""
import cmath
from typing import Optional

import numpy as np
import torch

from .AbstractGate import _Fixed, _Param, _cexp


class ZGate(_Fixed):
    _NAME, _DATA = 'Z', [[1, 0], [0, -1]]                      # ZGates.py:15-45


class RZGate(_Param):                                          # ZGates.py:48-84
    _NAME = 'RZ'

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        return self._mat([[_cexp(-self.theta / 2), 0], [0, _cexp(self.theta / 2)]])

    @staticmethod
    def _build_np(theta):
        return np.array([[cmath.exp(-0.5j * theta), 0], [0, cmath.exp(0.5j * theta)]], dtype=np.complex128)


class CZGate(_Fixed):                                          # ZGates.py:87-119
    _NAME, _SINGLE = 'CZ', False
    _DATA = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, -1]]


class RZZGate(_Param):                                         # ZGates.py:122-159
    _NAME, _SINGLE = 'RZZ', False

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        mi, pl = _cexp(-self.theta / 2), _cexp(self.theta / 2)
        return self._mat([[mi, 0, 0, 0], [0, pl, 0, 0], [0, 0, pl, 0], [0, 0, 0, mi]])
