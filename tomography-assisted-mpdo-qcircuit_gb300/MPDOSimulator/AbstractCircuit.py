"""Gate-queue circuit API (reference: MPDOSimulator/AbstractCircuit.py).

Gate methods only queue ``QuantumGate`` modules in ``self.layers``; nothing is
computed until ``evolve``.  Signatures follow the reference, including the
realNoise expansions of CX/CNOT/RXX/RYY/RZZ into ideal single-qubit rotations
around the measured CZ process (AbstractCircuit.py:221-301, 332-342).
"""
from abc import ABC, abstractmethod
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Union

import torch
from torch import Tensor, nn, pi

from .RealNoise import czExp_channel, cpExp_channel
from .Tools import select_device

CHIFILENAMES = {'CZ': {}, 'CP': {}}


def _info(x):
    return x.item() if isinstance(x, Tensor) else x


class QuantumCircuit(ABC, nn.Module):
    def __init__(self, noiseFiles: Optional[Dict[str, Dict[str, Any]]] = None, chi: Optional[int] = None,
                 kappa: Optional[int] = None, max_truncation_err: Optional[float] = None,
                 dtype=torch.complex64, device: Union[str, int] = 'cpu'):
        super().__init__()
        self.device = select_device(device)
        self.dtype = dtype
        self.chi = chi
        self.kappa = kappa
        self.max_truncation_err = max_truncation_err
        self.layers = nn.Sequential()
        self._oqs_list = []
        self.noiseTensorDict = {}
        self.unified, self.realNoise, self.idealNoise = False, False, False
        self.noiseFiles = noiseFiles if noiseFiles is not None else CHIFILENAMES
        self._initState = None
        self._vector = None
        self._stateNodes, self._dm, self._dmNodes = None, None, None
        self._samples, self._counts = None, None
        self._sequence = 0
        self._projectors_string = ['X', 'Y', 'Z']
        self._cz_expTensors, self._cp_expTensors = {}, {}

    def _load_exp_tensors(self):
        """AbstractCircuit.py:66-75."""
        self._cz_expTensors, self._cp_expTensors = {}, {}
        for key, fn in self.noiseFiles.get('CZ', {}).items():
            self._cz_expTensors[key] = czExp_channel(filename=fn).to(self.device, dtype=self.dtype)
        for key, fn in self.noiseFiles.get('CP', {}).items():
            self._cp_expTensors[key] = cpExp_channel(filename=fn).to(self.device, dtype=self.dtype)

    @dataclass
    class Group:
        history: List[int]
        start: int
        length: int

    @property
    def dm(self):
        return self._dm

    @property
    def samples(self):
        return self._samples

    @property
    def counts(self):
        return self._counts

    @property
    def initial_state(self):
        return self._initState

    @property
    def stateNodes(self):
        return self._stateNodes

    @property
    def dmNodes(self):
        return self._dmNodes

    @property
    def vector(self):
        return self._vector

    @abstractmethod
    def cal_vector(self):
        pass

    @abstractmethod
    def cal_dm(self):
        pass

    @abstractmethod
    def evolve(self, state):
        pass

    def _add_module(self, _gate: nn.Module, oqs: List, headline: str):
        self._oqs_list.append(oqs)
        self.layers.add_module(headline + f'-S{self._sequence}', _gate)
        self._sequence += 1

    def _kw(self):
        return dict(dtype=self.dtype, device=self.device)

    # -------------------------------------------------------------- 1q ---
    def _single(self, cls, oqs, _ideal, headline, *params):
        if isinstance(oqs, int):
            oqs = [oqs]
        self._add_module(cls(*params, _ideal, **self._kw()), oqs, headline.format(oqs))

    def i(self, oqs, _ideal=None):
        from .QuantumGates.SingleGates import IGate
        self._single(IGate, oqs, _ideal, 'I{}|None')

    def h(self, oqs, _ideal=None):
        from .QuantumGates.SingleGates import HGate
        self._single(HGate, oqs, _ideal, 'H{}|None')

    def x(self, oqs, _ideal=None):
        from .QuantumGates.XGates import XGate
        self._single(XGate, oqs, _ideal, 'X{}|None')

    def y(self, oqs, _ideal=None):
        from .QuantumGates.YGates import YGate
        self._single(YGate, oqs, _ideal, 'Y{}|None')

    def z(self, oqs, _ideal=None):
        from .QuantumGates.ZGates import ZGate
        self._single(ZGate, oqs, _ideal, 'Z{}|None')

    def rx(self, theta, oqs, _ideal=None):
        from .QuantumGates.XGates import RXGate
        self._single(RXGate, oqs, _ideal, ('RX{}|' + f'({_info(theta):.3f})').replace('.', ';'), theta)

    def ry(self, theta, oqs, _ideal=None):
        from .QuantumGates.YGates import RYGate
        self._single(RYGate, oqs, _ideal, ('RY{}|' + f'({_info(theta):.3f})').replace('.', ';'), theta)

    def rz(self, theta, oqs, _ideal=None):
        from .QuantumGates.ZGates import RZGate
        self._single(RZGate, oqs, _ideal, ('RZ{}|' + f'({_info(theta):.3f})').replace('.', ';'), theta)

    def s(self, oqs, _ideal=None):
        from .QuantumGates.PhaseGates import SGate
        self._single(SGate, oqs, _ideal, 'S{}|None')

    def sdg(self, oqs, _ideal=None):
        from .QuantumGates.PhaseGates import SDGGate
        self._single(SDGGate, oqs, _ideal, 'SDG{}|None')

    def t(self, oqs, _ideal=None):
        from .QuantumGates.PhaseGates import TGate
        self._single(TGate, oqs, _ideal, 'T{}|None')

    def p(self, theta, oqs, _ideal=None):
        from .QuantumGates.PhaseGates import PGate
        self._single(PGate, oqs, _ideal, ('P{}|' + f'({_info(theta):.3f})').replace('.', ';'), theta)

    def u1(self, theta, oqs, _ideal=None):
        from .QuantumGates.SingleGates import U1Gate
        self._single(U1Gate, oqs, _ideal, ('U1{}|' + f'({_info(theta):.3f})').replace('.', ';'), theta)

    def u2(self, phi, lam, oqs, _ideal=None):
        from .QuantumGates.SingleGates import U2Gate
        self._single(U2Gate, oqs, _ideal, ('U2{}|' + f'(P{_info(phi):3f})-(L{_info(lam):3f})').replace('.', ';'),
                     phi, lam)

    def u3(self, theta, phi, lam, oqs, _ideal=None):
        from .QuantumGates.SingleGates import U3Gate
        self._single(U3Gate, oqs, _ideal,
                     ('U3{}|' + f'(T{_info(theta):3f})-(P{_info(phi):3f})-(L{_info(lam):3f})').replace('.', ';'),
                     theta, phi, lam)

    def arbSingle(self, data: Tensor, oqs, _ideal=None):
        from .QuantumGates.SingleGates import ArbSingleGate
        self._single(ArbSingleGate, oqs, _ideal, 'ArbS{}|None', data)

    # -------------------------------------------------------------- 2q ---
    def _double(self, gate, oqs, headline):
        self._add_module(gate, oqs, headline)

    def rxx(self, theta, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.XGates import RXXGate
            self._double(RXXGate(theta, _ideal, **self._kw()), oqs, f'RXX{oqs}|({_info(theta):.3f})'.replace('.', ';'))
        else:
            self.h(oqs, True)
            self.cx(oq0, oq1)
            self.rz(theta, oq1, True)
            self.cx(oq0, oq1)
            self.h(oqs, True)

    def ryy(self, theta, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.YGates import RYYGate
            self._double(RYYGate(theta, _ideal, **self._kw()), oqs, f'RYY{oqs}|({_info(theta):.3f})'.replace('.', ';'))
        else:
            self.rx(torch.tensor(pi / 2), oqs, True)
            self.cx(oq0, oq1)
            self.rz(theta, oq1, True)
            self.cx(oq0, oq1)
            self.rx(-torch.tensor(pi / 2), oqs, True)

    def rzz(self, theta, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.ZGates import RZZGate
            self._double(RZZGate(theta, _ideal, **self._kw()), oqs, f'RZZ{oqs}|({_info(theta):.3f})'.replace('.', ';'))
        else:
            self.cx(oq0, oq1)
            self.rz(theta, oq1, True)
            self.cx(oq0, oq1)

    def xx_yy(self, theta, beta, control: int, target: int, _ideal=None):
        from .QuantumGates.DoubleGates import XXPlusYYGate
        oqs = [control, target]
        self._double(XXPlusYYGate(theta, beta, _ideal, **self._kw()), oqs,
                     f'XXPlusYYGate{oqs}|(P{_info(theta):3f})-(L{_info(beta):3f})'.replace('.', ';'))

    def cx(self, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.XGates import CXGate
            self._double(CXGate(_ideal, **self._kw()), oqs, f'CX{oqs}|None')
        else:
            self.ry(-torch.tensor(pi / 2), oq1, True)
            self.cz(oq0, oq1)
            self.ry(torch.tensor(pi / 2), oq1, True)

    def cy(self, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.YGates import CYGate
            self._double(CYGate(_ideal, **self._kw()), oqs, f'CY{oqs}|None')
        else:
            raise NotImplementedError('EXPCYGate is not implemented yet.')

    def cz(self, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.ZGates import CZGate
            self._double(CZGate(_ideal, **self._kw()), oqs, f'CZ{oqs}|None')
        else:
            from .QuantumGates.NoiseGates import CZEXPGate
            t = self._cz_expTensors.get(f'{oq0}{oq1}')
            if t is None:
                t = self._cz_expTensors.get(f'{oq1}{oq0}')
            self._double(CZEXPGate(t, **self._kw()), oqs, f'CZEXP{oqs}|None')

    def cnot(self, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.DoubleGates import CNOTGate
            self._double(CNOTGate(_ideal, **self._kw()), oqs, f'CNOT{oqs}|None')
        else:
            self.ry(-torch.tensor(pi / 2), oq1, True)
            self.cz(oq0, oq1)
            self.ry(torch.tensor(pi / 2), oq1, True)

    def swap(self, oq0: int, oq1: int, _ideal=None):
        from .QuantumGates.DoubleGates import SWAPGate
        self._double(SWAPGate(_ideal, **self._kw()), [oq0, oq1], f'SWAP{[oq0, oq1]}|None')

    def pswap(self, theta, oq0: int, oq1: int, _ideal=None):
        from .QuantumGates.DoubleGates import PSWAPGate
        self._double(PSWAPGate(theta, _ideal, **self._kw()), [oq0, oq1],
                     f'PSWAP{[oq0, oq1]}|({_info(theta):.3f})'.replace('.', ';'))

    def iswap(self, oq0: int, oq1: int, _ideal=None):
        from .QuantumGates.DoubleGates import ISWAPGate
        self._double(ISWAPGate(_ideal, **self._kw()), [oq0, oq1], f'ISWAP{[oq0, oq1]}|None')

    def cp(self, theta, oq0: int, oq1: int, _ideal=None):
        oqs = [oq0, oq1]
        if not self.realNoise or _ideal:
            from .QuantumGates.PhaseGates import CPGate
            self._double(CPGate(theta, _ideal, **self._kw()), oqs, f'CP{oqs}|({_info(theta):.3f})'.replace('.', ';'))
        else:
            from .QuantumGates.NoiseGates import CPEXPGate
            t = self._cp_expTensors.get(f'{oq0}{oq1}')
            if t is None:
                t = self._cp_expTensors.get(f'{oq1}{oq0}')
            self._double(CPEXPGate(t, **self._kw()), oqs, f'CPEXP{oqs}|None')

    def arbDouble(self, data: Tensor, oq1: int, oq2: int, _ideal=None):
        from .QuantumGates.DoubleGates import ArbDoubleGate
        self._double(ArbDoubleGate(data, _ideal, **self._kw()), [oq1, oq2], f'ArbD{[oq1, oq2]}|None')

    def ii(self, oq1: int, oq2: int, _ideal=None):
        from .QuantumGates.DoubleGates import IIGate
        self._double(IIGate(_ideal, **self._kw()), [oq1, oq2], f'II{[oq1, oq2]}|None')

    # ---------------------------------------------------------- layers ---
    def truncate(self):
        """AbstractCircuit.py:483-490."""
        from .QuantumGates.AbstractGate import Truncate
        self._oqs_list.append([None])
        self.layers.append(Truncate())

    def barrier(self):
        from .QuantumGates.AbstractGate import Barrier
        self._oqs_list.append([None])
        self.layers.append(Barrier())

    def reset0(self, oqs):
        from .QuantumGates.SingleGates import Reset0
        oqs = [oqs] if isinstance(oqs, int) else oqs
        self._add_module(Reset0(**self._kw()), oqs, f'Reset;0{oqs}|None')

    def reset1(self, oqs):
        from .QuantumGates.SingleGates import Reset1
        oqs = [oqs] if isinstance(oqs, int) else oqs
        self._add_module(Reset1(**self._kw()), oqs, f'Reset;1{oqs}|None')

    def measure(self, oqs, orientations=None):
        """AbstractCircuit.py:519-532: basis-change gates MeasureX/Y (Z is a no-op)."""
        from .QuantumGates.SingleGates import MeasureX, MeasureY, MeasureZ
        oqs = [oqs] if isinstance(oqs, int) else oqs
        orientations = orientations or [2] * len(oqs)
        orientations = [orientations] if isinstance(orientations, int) else orientations
        mm = {0: MeasureX, 1: MeasureY, 2: MeasureZ}
        for oq, ori in zip(oqs, orientations):
            if ori not in mm:
                raise ValueError('Orientation beyond the settings.')
            self._add_module(mm[ori](**self._kw()), [oq], f'Measure;{oq}|Orientation;{ori}')
