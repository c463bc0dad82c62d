"""Initial states, dense-matrix utilities and bookkeeping helpers
(reference: MPDOSimulator/Tools.py).

``create_ket*Series`` return one ``QubitNode`` per qubit (a physical-leg-only
node, as the reference's ``tn.Node`` list).  ``connected=True`` -- an
extension -- links neighbours by dimension-1 bonds, so truncate() layers act
from the first layer instead of waiting for every pair to have met a 2q gate.
"""
import itertools
import warnings
from collections import Counter
from functools import reduce
from typing import Dict, List, Optional, Union

import numpy as np
import torch
from torch import Tensor

__all__ = ['create_ket0Series', 'create_ket1Series', 'create_ketPlusSeries', 'create_ketMinusSeries',
           'create_ketRandomSeries', 'create_ketHadamardSeries', 'plot_histogram', 'plot_histogram_multiBars',
           'density2prob',
           'select_device', 'tc_expect', 'EdgeName2AxisName', 'count_item', 'cal_fidelity',
           'random_measurementScheme', 'QubitNode']

PUBLIC_SQRT2 = 1 / np.sqrt(2)


class QubitNode:
    """A site of an MPDO.  Before evolution: the product-state vector with axis
    ``physics_k``.  After evolution the circuit hands out nodes whose
    ``tensor`` is read lazily from the GPU with axes
    (bond_{k-1}_k, physics_k, I_k, bond_k_{k+1})."""

    def __init__(self, tensor: Optional[Tensor], name: str, axis_names: List[str], connected: bool = False,
                 chain=None, index: Optional[int] = None, dtype=None, device='cpu'):
        self._tensor = tensor
        self.name = name
        self.axis_names = list(axis_names)
        self.connected = connected
        self._chain, self._index = chain, index
        self._dtype, self._device = dtype, device

    @property
    def tensor(self) -> Tensor:
        if self._chain is not None:
            # copied device to device from the engine's site buffer (no host copy)
            t = self._chain.site_tensor(self._index)
            return t.to(dtype=self._dtype or t.dtype, device=self._device)
        return self._tensor

    def set_tensor(self, t: Tensor) -> None:
        self._tensor = t
        self._chain = None

    @property
    def shape(self):
        if self._chain is not None:
            return tuple(self._chain.site_dims(self._index))
        return tuple(self._tensor.shape)

    def __repr__(self):
        return f'QubitNode({self.name}, axes={self.axis_names}, shape={self.shape})'


def EdgeName2AxisName(_nodes):
    """Axis names follow the edge names already (reference Tools.py:44-72
    renames TensorNetwork axes after every operation); kept for API parity."""
    return None


def _series(qnumber, vec, dtype, device, connected):
    assert qnumber > 0
    return [QubitNode(vec.clone(), f'qubit_{i}', [f'physics_{i}'], connected=connected)
            for i in range(qnumber)]


def ket0(dtype, device='cpu'):
    return torch.tensor([1. + 0.j, 0. + 0.j], dtype=dtype, device=device)


def ket1(dtype, device='cpu'):
    return torch.tensor([0. + 0.j, 1. + 0.j], dtype=dtype, device=device)


def ket_plus(dtype, device='cpu'):
    return PUBLIC_SQRT2 * torch.tensor([1., 1.], dtype=dtype, device=device)


ket_hadamard = ket_plus


def ket_minus(dtype, device='cpu'):
    return PUBLIC_SQRT2 * torch.tensor([1., -1.], dtype=dtype, device=device)


def create_ket0Series(qnumber: int, dtype=torch.complex64, device='cpu', connected: bool = False) -> list:
    return _series(qnumber, ket0(dtype, device), dtype, device, connected)


def create_ket1Series(qnumber: int, dtype=torch.complex64, device='cpu', connected: bool = False) -> list:
    return _series(qnumber, ket1(dtype, device), dtype, device, connected)


def create_ketHadamardSeries(qnumber: int, dtype=torch.complex64, device='cpu', connected: bool = False) -> list:
    return _series(qnumber, ket_hadamard(dtype, device), dtype, device, connected)


def create_ketPlusSeries(qnumber: int, dtype=torch.complex64, device='cpu', connected: bool = False) -> list:
    return _series(qnumber, ket_plus(dtype, device), dtype, device, connected)


def create_ketMinusSeries(qnumber: int, dtype=torch.complex64, device='cpu', connected: bool = False) -> list:
    return _series(qnumber, ket_minus(dtype, device), dtype, device, connected)


def create_ketRandomSeries(qnumber: int, tensor: Tensor, dtype=torch.complex64, device='cpu',
                           connected: bool = False) -> list:
    return _series(qnumber, tensor.to(dtype=dtype, device=device), dtype, device, connected)


def tc_expect(oper, state):
    """Tools.py:201-239."""
    def one(o, s):
        if s.dim() == 1:
            return torch.einsum('i, ij, j', s.conj(), o, s)
        if s.dim() == 2:
            return torch.trace(torch.matmul(o, s))
        raise ValueError('State must be a vector or matrix.')

    if isinstance(oper, Tensor) and isinstance(state, Tensor):
        return one(oper, state)
    if isinstance(oper, list) and isinstance(state, Tensor):
        return torch.tensor([one(o, state) for o in oper], dtype=state.dtype)
    if isinstance(state, list):
        return torch.tensor([one(oper, x) for x in state], dtype=oper.dtype)
    raise TypeError('Arguments must be torch.Tensors or lists thereof')


def density2prob(rho_in: Tensor, bases: Optional[Dict] = None, tol: Optional[float] = None,
                 _dict: Optional[bool] = True):
    """Tools.py:242-273: |<i|rho|i>| normalised by their sum."""
    qn = int(np.log2(rho_in.shape[0]))
    if bases is None:
        probs = torch.abs(torch.diagonal(rho_in)).detach().cpu().double().numpy()
        names = [''.join(b) for b in itertools.product('01', repeat=qn)]
    else:
        basis, names = bases['Bases'], bases['BasesName']
        probs = np.array([abs(tc_expect(rho_in, b.view(-1))).item() for b in basis])
    total = probs.sum()
    if _dict:
        return {n: p / total for n, p in zip(names, probs) if tol is None or p >= tol}
    return probs / total


def plot_histogram(*args, **kwargs):
    """Plotting needs matplotlib, which is not part of this engine."""
    raise ImportError('plot_histogram needs matplotlib; plotting is not part of the GB300 engine')


def plot_histogram_multiBars(*args, **kwargs):
    """Tools.py:339-449 plots with matplotlib, which is not part of this engine."""
    raise ImportError('plot_histogram_multiBars needs matplotlib; plotting is not part of the GB300 engine')


def select_device(device: Optional[Union[str, int]] = None):
    """Tools.py:452-463."""
    if isinstance(device, str):
        return device
    if torch.cuda.is_available():
        return 'cuda:0' if device is None else f'cuda:{device}'
    warnings.warn('CUDA is not available, use CPU instead.')
    return 'cpu'


def gates_list(N: int, basis_gates: Optional[List[str]] = None) -> List[str]:
    """Tools.py:466-485."""
    basis_gates = basis_gates or ['I', 'X', 'Y', 'Z']
    return [''.join(g) for g in itertools.product(basis_gates, repeat=N)]


def name2matrix(operation_name: str, dtype=torch.complex64, device='cpu'):
    """Tools.py:488-509 (Y is -iY, a real matrix)."""
    ops = {'I': torch.eye(2, dtype=dtype, device=device),
           'X': torch.tensor([[0, 1], [1, 0]], dtype=dtype, device=device),
           'Y': -1j * torch.tensor([[0, -1j], [1j, 0]], dtype=dtype, device=device),
           'Z': torch.tensor([[1, 0], [0, -1]], dtype=dtype, device=device)}
    return reduce(torch.kron, [ops[c] for c in operation_name])


def sqrt_matrix(density_matrix: Tensor) -> Tensor:
    """Tools.py:512-525."""
    evs, vecs = torch.linalg.eigh(density_matrix)
    evs = torch.where(evs > 1e-10, evs, torch.zeros((), dtype=evs.dtype, device=evs.device))
    return vecs @ torch.diag(torch.sqrt(evs)).to(vecs.dtype) @ vecs.conj().transpose(-2, -1)


def cal_fidelity(rho: Tensor, sigma: Tensor) -> Tensor:
    """Uhlmann fidelity (Tools.py:528-551)."""
    if rho.shape != sigma.shape:
        raise ValueError('The shape of rho and sigma should be equal.')
    if rho.shape[0] != rho.shape[1] or rho.shape[0] != sigma.shape[1]:
        raise ValueError('The shape of rho and sigma should be square.')
    sr = sqrt_matrix(rho)
    evs = torch.linalg.eigvalsh(sr @ sigma @ sr)
    evs = torch.where(evs > 1e-12, evs, torch.zeros((), dtype=evs.dtype, device=evs.device))
    return torch.sum(torch.sqrt(evs)) ** 2


def count_item(data):
    """Tools.py:554-570."""
    def key(x):
        if isinstance(x[0], tuple):
            return int(''.join(str(int(v)) for v in x[0]))
        if isinstance(x[0], str):
            return x[0]
        return int(x[0])
    counted = dict(Counter([tuple(i) if isinstance(i, list) else i for i in data]))
    return dict(sorted(counted.items(), key=key))


def random_measurementScheme(qnumber: int, amount: int) -> List[List[int]]:
    """Tools.py:573-584."""
    return np.random.randint(0, 3, size=(amount, qnumber)).tolist()
