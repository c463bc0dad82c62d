"""Single-qubit gates (reference: QuantumGates/SingleGates.py)."""
import cmath
import math
from typing import Optional
from warnings import warn

import numpy as np
import torch
from torch import Tensor

from .AbstractGate import QuantumGate, _Fixed, _Param, _cexp

_S2 = 1 / math.sqrt(2)


class IGate(_Fixed):
    _NAME, _DATA = 'I', [[1, 0], [0, 1]]                       # SingleGates.py:17-47


class HGate(_Fixed):
    _NAME, _DATA = 'H', [[_S2, _S2], [_S2, -_S2]]              # SingleGates.py:50-80


class U1Gate(_Param):                                          # SingleGates.py:83-119
    _NAME = 'U1'

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        return self._mat([[1, 0], [0, _cexp(self.theta)]])


class U2Gate(_Param):                                          # SingleGates.py:122-159
    _NAME = 'U2'

    def __init__(self, phi, lam, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.phi, self.lam = self._check_Para_Tensor(phi, lam)
        self.para = [self.phi, self.lam]

    def _build(self):
        lm, pm = _cexp(self.lam), _cexp(self.phi)
        return self._mat([[_S2, -lm * _S2], [pm * _S2, lm * pm * _S2]])


class U3Gate(_Param):                                          # SingleGates.py:162-201
    _NAME = 'U3'

    def __init__(self, theta, phi, lam, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta, self.phi, self.lam = self._check_Para_Tensor(theta, phi, lam)
        self.para = [self.theta, self.phi, self.lam]

    def _build(self):
        lm, pm = _cexp(self.lam), _cexp(self.phi)
        c, s = torch.cos(self.theta / 2), torch.sin(self.theta / 2)
        return self._mat([[c, -lm * s], [pm * s, lm * pm * c]])

    @staticmethod
    def _build_np(theta, phi, lam):
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        el, ep = cmath.exp(1j * lam), cmath.exp(1j * phi)
        return np.array([[c, -el * s], [ep * s, el * ep * c]], dtype=np.complex128)


class ArbSingleGate(QuantumGate):                              # SingleGates.py:204-237
    def __init__(self, tensor: Tensor, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self._matrix = tensor.to(dtype=self.dtype, device=self.device)

    @property
    def name(self):
        return 'ArbSingleGate'

    @property
    def tensor(self):
        if self._matrix.shape != (2, 2):
            warn('You are probably adding a noisy single qubit gate, current shape is {}'.format(self._matrix.shape))
        return self._matrix.reshape(2, 2, -1).squeeze()

    @property
    def rank(self):
        return 2

    @property
    def dimension(self):
        return [2, 2]

    @property
    def single(self) -> bool:
        return True

    @property
    def variational(self) -> bool:
        return False


class _Measure(_Fixed):
    def __init__(self, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=True, dtype=dtype, device=device)


class MeasureX(_Measure):
    _NAME, _DATA = 'MeasureX', [[_S2, _S2], [_S2, -_S2]]        # SingleGates.py:240-271


class MeasureY(_Measure):
    _NAME, _DATA = 'MeasureY', [[_S2, -1j * _S2], [_S2, 1j * _S2]]   # SingleGates.py:274-305


class MeasureZ(_Measure):
    _NAME, _DATA = 'MeasureZ', [[1, 0], [0, 1]]                # SingleGates.py:308-339


class Reset0(_Measure):
    _NAME, _DATA = 'Reset0', [[1, 0], [0, 0]]                  # SingleGates.py:342-373


class Reset1(_Measure):
    _NAME, _DATA = 'Reset1', [[0, 0], [0, 1]]                  # SingleGates.py:376-407
