"""Kraus tensors of the noise channels (reference: MPDOSimulator/NoiseChannel.py).

Layouts match the reference: (2, 2, K) = [out, in, k] for one qubit,
(2, 2, 2, 2, K) = [out0, out1, in0, in1, k] for two.  The attributes
``decayTensor``, ``dephasingTensor``, ``dpCTensor``, ``dpCTensor2`` and
``apdeCTensor`` may be overwritten by the user before ``evolve``.
"""
import math
import warnings
from typing import Optional, Union

import numpy as np
import torch

from .ChipInfo import ChipInformation
from .Tools import select_device

_PAULI = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]])]


class NoiseChannel:
    def __init__(self, chip: Optional[str] = None, dtype=torch.complex64, device: Union[str, int] = 'cpu'):
        self.dtype = dtype
        self.device = select_device(device)
        self.chip = getattr(ChipInformation(), chip or 'worst')()
        self.bath_rate = self.chip.bath_rate
        self.decay_rate = self.chip.decay_rate
        self.dephasing_rate = self.chip.dephasing_rate
        self.T1 = self.chip.T1
        self.T2 = self.chip.T2
        self.GateTime = self.chip.gateTime
        self.dpc_errorRate = self.chip.dpc_errorRate
        self.decayTensor = self.decay(self.decay_rate, self.GateTime)
        self.dephasingTensor = self.dephasing(self.dephasing_rate, self.GateTime)
        self.dpCTensor = self.depolarization_noise_channel(p=self.dpc_errorRate)
        self.dpCTensor2 = self.depolarization_noise_channel(p=self.dpc_errorRate, qn=2)
        self.apdeCTensor = self.amp_phase_damping_error(time=self.GateTime, T1=self.T1, T2=self.T2)

    def _t(self, a):
        return torch.as_tensor(np.asarray(a, dtype=np.complex128), dtype=self.dtype, device=self.device)

    def depolarization_noise_channel(self, p: float, qn: int = 1) -> torch.Tensor:
        """(1 - (4^n-1)p/4^n) rho + p/4^n sum_P P rho P  (NoiseChannel.py:51-91)."""
        if not 0 <= p <= 1:
            raise ValueError('Probability p must be in the range [0, 1].')
        d = 4 ** qn
        w = [math.sqrt(1 - (d - 1) * p / d)] + [math.sqrt(p / d)] * (d - 1)
        ops = list(_PAULI)
        for _ in range(qn - 1):
            ops = [np.kron(e, b) for e in ops for b in _PAULI]
        t = np.stack(ops) * np.asarray(w)[:, None, None]
        return self._t(np.transpose(t, (1, 2, 0)).reshape([2] * (2 * qn) + [d]))

    def amp_phase_damping_error(self, time: float, T1: float, T2: float) -> torch.Tensor:
        """NoiseChannel.py:93-142."""
        if time < 0 or T1 <= 0 or T2 <= 0:
            raise ValueError('The time, T1, T2 must be greater than or equal to 0, '
                             'for some special cases time = 0 is allowed.')
        if time == 0:
            warnings.warn('The time is 0, which means the noise is not applied.')
        t2p = 2 * T1 * T2 / (2 * T1 - T2)
        p1 = 1 - math.exp(-time / T1)
        p2 = 1 - math.exp(-time / t2p)
        k = np.array([[[1, 0], [0, math.sqrt(1 - (p1 + p2))]], [[0, 0], [0, math.sqrt(p2)]],
                      [[0, math.sqrt(p1)], [0, 0]]])
        return self._t(np.transpose(k, (1, 2, 0)))

    def decay(self, gamma: float, gate_time: float):
        """Amplitude damping, NoiseChannel.py:144-155."""
        if gate_time <= 0:
            raise ValueError('The gate time must be greater than 0, or set the gate to IDEAL.')
        p = 1 - math.exp(-self.bath_rate * gamma * gate_time)
        k = np.array([[[1, 0], [0, math.sqrt(1 - p)]], [[0, math.sqrt(p)], [0, 0]]])
        return self._t(np.transpose(k, (1, 2, 0)))

    def dephasing(self, gamma: float, gate_time: float):
        """NoiseChannel.py:157-170."""
        if gate_time <= 0:
            raise ValueError('The gate time must be greater than 0, or set the gate to IDEAL.')
        p = 1 - math.exp(-self.bath_rate * gamma * gate_time)
        sp, s1 = math.sqrt(p), math.sqrt(1 - p)
        k = np.array([[[s1, 0], [0, s1]], [[sp, 0], [0, 0]], [[0, 0], [0, sp]]])
        return self._t(np.transpose(k, (1, 2, 0)))
