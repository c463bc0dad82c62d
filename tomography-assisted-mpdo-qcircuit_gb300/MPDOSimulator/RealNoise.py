"""Experimental process (chi) matrix -> Kraus tensor of a noisy two-qubit gate
(reference: MPDOSimulator/RealNoise.py)."""
import os
from typing import Dict, List, Optional, Union

import numpy as np
import torch

from .Tools import gates_list, name2matrix

__all__ = ['czExp_channel', 'cpExp_channel']


def readExpChi(filename: Optional[str] = None):
    """RealNoise.py:22-32: .mat (key 'exp') or .npz (key 'chi')."""
    if filename is None:
        raise FileNotFoundError('No file found.')
    if '.mat' in filename:
        from scipy.io import loadmat
        return loadmat(filename)['exp']
    if '.npz' in filename:
        return np.load(filename)['chi']
    raise TypeError('Current file-type is not supported.')


def noisyTensor(chi, gate_factor: Optional[Dict] = None, dtype=torch.complex64,
                device: Union[int, str] = 'cpu') -> List[torch.Tensor]:
    """RealNoise.py:35-161: Kraus operators E_i = sqrt(d_i) sum_j U_ji P_j from
    the eigen-decomposition of the chi matrix (descending complex sort,
    |lambda| > 1e-12, coefficients below 1e-12 zeroed).  Returns a list of
    (2,2,2,2) tensors."""
    if gate_factor is None:
        s, u = np.linalg.eig(chi)
        idx = s.argsort()[::-1]
        s, u = s[idx], u[:, idx]
        count = int(np.sum(np.abs(s) > 1e-12))
        nq = int(round(np.log10(chi.shape[0]) / np.log10(4)))
        names = gates_list(nq)
        factors = []
        for i in range(count):
            e = u[:, i] * np.sqrt(s[i] + 0j)
            e = np.where(np.abs(e) < 1e-12, 0, e)
            factors.append({names[j]: e[j] for j in range(len(names)) if e[j] != 0})
    else:
        nested = any(isinstance(v, dict) for v in gate_factor.values())
        factors = list(gate_factor.values()) if nested else [gate_factor]
    out = []
    for f in factors:
        t = torch.zeros((2, 2, 2, 2), dtype=dtype, device=device)
        for name, val in f.items():
            t = t + (torch.tensor(val, dtype=dtype, device=device) *
                     name2matrix(name, dtype=dtype, device=device)).reshape(2, 2, 2, 2)
        out.append(t)
    return out


def _exp_channel(filename, dtype, device):
    if not os.path.exists(filename):
        raise FileNotFoundError(f'chi-matrix file {filename!r} not found; the measured default chi matrices '
                                '(chi/czDefault.mat, chi/cpDefault.mat) are the reference\'s data and do not '
                                'ship with this package: pass the file (chiFileDict / filename=)')
    chi = readExpChi(filename=filename)
    t = torch.stack(noisyTensor(chi))
    return torch.einsum('ijlmn -> jlmni', t).to(dtype=dtype, device=device)


def czExp_channel(filename: Optional[str] = None, dtype=torch.complex64, device: Union[int, str] = 'cpu'):
    """RealNoise.py:164-170."""
    if filename is None:
        filename = os.path.join(os.path.dirname(__file__), 'chi', 'czDefault.mat')
    return _exp_channel(filename, dtype, device)


def cpExp_channel(filename: Optional[str] = None, dtype=torch.complex64, device: Union[int, str] = 'cpu'):
    """RealNoise.py:173-179."""
    if filename is None:
        filename = os.path.join(os.path.dirname(__file__), 'chi', 'cpDefault.mat')
    return _exp_channel(filename, dtype, device)
