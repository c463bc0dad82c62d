"""Experimental noisy two-qubit processes (reference: QuantumGates/NoiseGates.py).
The tensor carries its Kraus leg last: (2, 2, 2, 2, K)."""
import os
import warnings
from typing import Optional

import torch
from torch import Tensor

from .AbstractGate import QuantumGate

_CHI_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'chi')


class _ExpGate(QuantumGate):
    _NAME = ''
    _DEFAULT = ''

    def __init__(self, tensor: Optional[Tensor] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(dtype=dtype, device=device)
        self.ideal = False
        self._matrix = tensor

    @property
    def name(self):
        return self._NAME

    @property
    def tensor(self):
        if self._matrix is None:
            warnings.warn(f'No (sufficient) {self._NAME[:2]} input files, use default tensor.')
            from ..RealNoise import czExp_channel
            path = os.path.join(_CHI_DIR, self._DEFAULT)
            if not os.path.exists(path):
                raise FileNotFoundError(f'default chi matrix {self._DEFAULT} is not available; pass a chi file')
            return czExp_channel(filename=path).to(dtype=self.dtype, device=self.device)
        return self._matrix.to(dtype=self.dtype, device=self.device)

    @property
    def rank(self):
        return 5

    @property
    def dimension(self):
        return [[2, 2], [2, 2], [16]]

    @property
    def single(self) -> bool:
        return False

    @property
    def variational(self) -> bool:
        return False


class CZEXPGate(_ExpGate):                                     # NoiseGates.py:15-52
    _NAME, _DEFAULT = 'CZEXP', 'czDefault.mat'


class CPEXPGate(_ExpGate):                                     # NoiseGates.py:55-92
    _NAME, _DEFAULT = 'CPEXP', 'cpDefault.mat'
