"""Readout on the doubled (ket x conj) network (reference: MPDOSimulator/dmOperations.py).

``DMNodes`` stands for the reference's list of 2n TensorNetwork nodes: it
keeps the GPU chain and the set of qubits whose physical legs are traced.
All contractions run on the GPU through the engine's environment sweeps.
"""
from typing import List, Optional, Union

import numpy as np
import torch
from torch import Tensor

PAULI_DICT = {0: torch.tensor([[0, 1], [1, 0]]), 1: torch.tensor([[0, -1j], [1j, 0]]),
              2: torch.tensor([[1, 0], [0, -1]])}


class DMNodes:
    def __init__(self, chain, qnumber: int, dtype, device):
        self.chain, self.qnumber, self.dtype, self.device = chain, qnumber, dtype, device
        self.traced = set()

    def __len__(self):
        return 2 * self.qnumber

    def trace_out(self, idx):
        idx = [idx] if isinstance(idx, int) else list(idx)
        if idx and max(idx) >= self.qnumber:
            raise ValueError(f'Reduced index should not be larger than the qubit number. {max(idx)}-{self.qnumber}')
        self.traced.update(idx)

    def kept(self) -> List[int]:
        return [q for q in range(self.qnumber) if q not in self.traced]


def reduce_dmNodes(qubits_nodes, conj_qubits_nodes=None, residual_index=None, reduced_index=None):
    """dmOperations.py:18-37: trace the physical legs of ``reduced_index``."""
    if reduced_index is None:
        return None
    nodes = qubits_nodes if isinstance(qubits_nodes, DMNodes) else conj_qubits_nodes
    nodes.trace_out(reduced_index)


def _trace_product(a: np.ndarray, b: np.ndarray) -> float:
    """Re Tr(a b) = Re sum_ij a_ij b_ji without forming the product (O(d^2),
    not O(d^3), for the 4096 x 4096 matrices of twelve kept qubits)."""
    return float(np.sum(a * b.T).real)


def trace_rho(dmNodes: DMNodes) -> Tensor:
    """dmOperations.py:40-48: Tr rho (real part)."""
    return torch.tensor(dmNodes.chain.expect_ops({}), dtype=torch.float64)


def trace_rho_rho(dmNodes_0: DMNodes, dmNodes_1: Optional[DMNodes] = None) -> Tensor:
    """dmOperations.py:51-66: Tr(rho_0 rho_1) over the untraced qubits (up to
    12 of them through the reduced density matrices, beyond that by the
    engine's four-layer environment sweep)."""
    d1 = dmNodes_1 if dmNodes_1 is not None else dmNodes_0
    if d1.qnumber != dmNodes_0.qnumber:
        raise ValueError('Density matrices must have the same number of nodes.')
    keep = dmNodes_0.kept()
    if d1.kept() != keep:
        raise ValueError('Density matrices should have the same untraced qubits.')
    if len(keep) > 12:
        # four-layer environment sweep on the GPU, no density matrix formed
        return torch.tensor(dmNodes_0.chain.trace_rho_rho(d1.chain, keep), dtype=torch.float64)
    r0 = dmNodes_0.chain.reduced_dm(keep)
    r1 = d1.chain.reduced_dm(keep)
    return torch.tensor(_trace_product(r0, r1), dtype=torch.float64)


def trace_rho2(dmNodes: DMNodes) -> Tensor:
    return trace_rho_rho(dmNodes)


def trace_composited_rho(*dmNodes: DMNodes) -> Tensor:
    """dmOperations.py:73-87."""
    return sum(trace_rho_rho(d) for d in dmNodes)


def trace_composited_rho2(*dmNodes: DMNodes) -> Tensor:
    """dmOperations.py:90-132: Tr[(sum_i rho_i)^2] / slices^2."""
    n = len(dmNodes)
    keep = dmNodes[0].kept()
    if any(d.kept() != keep for d in dmNodes):
        raise ValueError('Density matrices should have same number of un-traced nodes.')
    if len(keep) > 12:
        # as the reference beyond 12 qubits: diagonal terms plus twice the cross terms
        diag = sum(d.chain.trace_rho_rho(d.chain, keep) for d in dmNodes)
        cross = sum(dmNodes[i].chain.trace_rho_rho(dmNodes[k].chain, keep)
                    for i in range(n) for k in range(i + 1, n))
        return torch.tensor((diag + 2 * cross) / n ** 2, dtype=torch.float64)
    rho = sum(d.chain.reduced_dm(keep) for d in dmNodes)
    return torch.tensor(_trace_product(rho, rho) / n ** 2, dtype=torch.float64)


def expect(dmNodes: DMNodes, observables: Union[Tensor, List[Tensor]], oqs) -> List[Tensor]:
    """dmOperations.py:135-171: Re Tr(rho O) per observable, O given on the
    qubits ``oq`` in the listed order; all other qubits traced."""
    qn = dmNodes.qnumber
    oqs = [oqs] if isinstance(oqs, int) else oqs
    observables = [observables] if isinstance(observables, Tensor) else observables
    out = []
    for j, (obs, oq) in enumerate(zip(observables, oqs)):
        oq = [oq] if isinstance(oq, int) else list(oq)
        m = len(oq)
        try:
            o = obs.reshape([2] * 2 * m)
        except RuntimeError:
            raise ValueError(f'Shape of the No.{j} obs is not valid, which is: {obs.shape}.')
        if m > qn:
            raise ValueError(f'Dim of No.{j} - oqs: {m} exceeds the system size.')
        order = sorted(oq)
        perm = [oq.index(q) for q in order] + [m + oq.index(q) for q in order]
        o = o.permute(*perm).reshape(2 ** m, 2 ** m).detach().cpu().numpy().astype(np.complex128)
        rho = dmNodes.chain.reduced_dm(order)
        out.append(torch.tensor(_trace_product(rho, o), dtype=torch.float64))
    return out


def pauli_expect(dmNodes: DMNodes, observables, oqs) -> Tensor:
    """dmOperations.py:174-201: Re Tr(rho prod_j P_j) with P in {0: X, 1: Y, 2: Z}."""
    oqs = [oqs] if isinstance(oqs, int) else list(oqs)
    observables = [observables] if isinstance(observables, int) else list(observables)
    ops = {q: PAULI_DICT[o].numpy().astype(np.complex128) for o, q in zip(observables, oqs)}
    return torch.tensor(dmNodes.chain.expect_ops(ops), dtype=torch.float64)
