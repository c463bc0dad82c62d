"""Exact dense density-matrix simulator (n <= 10): the physics pin.

TEST INFRASTRUCTURE ONLY.  Applies the same Kraus channels as the MPDO path to
rho (2^n x 2^n, qubit 0 most significant, complex128) with no truncation, so an
MPDO run whose chi and kappa never bind must agree with it to rounding.
"""
from __future__ import annotations

import torch

from .mpdo_oracle import orient_2q


def zero_state(n: int, vectors=None) -> torch.Tensor:
    psi = torch.ones(1, dtype=torch.complex128)
    for q in range(n):
        v = torch.tensor([1, 0], dtype=torch.complex128) if vectors is None else \
            torch.as_tensor(vectors[q], dtype=torch.complex128)
        psi = torch.kron(psi, v)
    return torch.outer(psi, psi.conj())


def apply_channel(rho: torch.Tensor, n: int, qubits, kraus: torch.Tensor) -> torch.Tensor:
    """rho -> sum_k K_k rho K_k^dagger on ``qubits`` (ascending, adjacent)."""
    m = len(qubits)
    if kraus.dim() == 2 * m:
        kraus = kraus.unsqueeze(-1)
    K = kraus.shape[-1]
    ops = kraus.to(torch.complex128).reshape(2 ** m, 2 ** m, K)
    t = rho.reshape([2] * (2 * n))
    q0 = qubits[0]
    # move target ket axes to front, bra axes after them
    ket = list(qubits)
    bra = [n + q for q in qubits]
    rest = [i for i in range(2 * n) if i not in ket + bra]
    t = t.permute(*(ket + bra + rest)).reshape(2 ** m, 2 ** m, -1)
    out = torch.einsum('xak,abR,ybk->xyR', ops, t, ops.conj())
    out = out.reshape([2] * (2 * m) + [2] * (2 * n - 2 * m))
    inv = [0] * (2 * n)
    for pos, ax in enumerate(ket + bra + rest):
        inv[ax] = pos
    del q0
    return out.permute(*inv).reshape(2 ** n, 2 ** n)


def run(n: int, ops, vectors=None) -> torch.Tensor:
    rho = zero_state(n, vectors)
    for op in ops:
        if op[0] == '1q':
            rho = apply_channel(rho, n, [op[1]], op[2])
        elif op[0] == '2q':
            i, t = orient_2q(op[1], op[2], op[3])
            rho = apply_channel(rho, n, [i, i + 1], t)
    return rho
