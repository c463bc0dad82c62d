"""Two-qubit gates (reference: QuantumGates/DoubleGates.py)."""
from typing import Optional
from warnings import warn

import torch
from torch import Tensor

from .AbstractGate import QuantumGate, _Fixed, _Param, _cexp


class IIGate(_Fixed):                                          # DoubleGates.py:15-47
    _NAME, _SINGLE = 'II', False
    _DATA = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]]


class CNOTGate(_Fixed):                                        # DoubleGates.py:50-82
    _NAME, _SINGLE = 'CNOT', False
    _DATA = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]


class ISWAPGate(_Fixed):                                       # DoubleGates.py:85-117
    _NAME, _SINGLE = 'ISWAP', False
    _DATA = [[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]]


class SWAPGate(_Fixed):                                        # DoubleGates.py:120-152
    _NAME, _SINGLE = 'SWAP', False
    _DATA = [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]]


class PSWAPGate(_Param):                                       # DoubleGates.py:155-190
    # the reference reports the name 'SWAP' (DoubleGates.py:167)
    _NAME, _SINGLE = 'SWAP', False

    def __init__(self, theta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.para = self.theta

    def _build(self):
        c, s = torch.cos(self.theta), torch.sin(self.theta)
        return self._mat([[1, 0, 0, 0], [0, c, s, 0], [0, s, c, 0], [0, 0, 0, 1]])


class ArbDoubleGate(QuantumGate):                              # DoubleGates.py:193-226
    def __init__(self, matrix: Tensor, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self._matrix = matrix.to(dtype=self.dtype, device=self.device)

    @property
    def name(self):
        return 'ArbDoubleGate'

    @property
    def tensor(self):
        if self._matrix.shape != (2, 2, 2, 2):
            warn('You are probably adding a noisy double qubit gate, current shape is {}'.format(self._matrix.shape))
        return self._matrix.reshape(2, 2, 2, 2, -1).squeeze()

    @property
    def rank(self):
        return 4

    @property
    def dimension(self):
        return [[2, 2], [2, 2]]

    @property
    def single(self) -> bool:
        return False

    @property
    def variational(self) -> bool:
        return True


class XXPlusYYGate(_Param):                                    # DoubleGates.py:229-270
    # the reference reports the name 'SWAP' (DoubleGates.py:243)
    _NAME, _SINGLE = 'SWAP', False

    def __init__(self, theta, beta, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)
        self.theta = self._check_Para_Tensor(theta)
        self.beta = self._check_Para_Tensor(beta)
        self.para = [self.theta, self.beta]

    def _build(self):
        c, s = torch.cos(self.theta / 2), -1j * torch.sin(self.theta / 2)
        return self._mat([[1, 0, 0, 0], [0, c, s * _cexp(self.beta), 0],
                          [0, s * _cexp(-self.beta), c, 0], [0, 0, 0, 1]])
