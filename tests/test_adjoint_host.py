"""Host logic of the GPU adjoint (no device needed): the Pauli-sum
matrix-product operator that carries the loss, and the differentiable gate /
channel builders of the gradient workload against the oracle's."""
import numpy as np
import pytest
import torch

from oracle import adjoint as OA, mpdo_oracle as O

AD = pytest.importorskip('mpdo_gb300.adjoint')


def _dense_from_mpo(n, dims, W):
    off, out = 0, np.ones((1, 1, 1), dtype=np.complex128)      # [D][row][col]
    for k in range(n):
        w = W[off: off + dims[k] * dims[k + 1] * 4].reshape(dims[k], dims[k + 1], 2, 2)
        off += dims[k] * dims[k + 1] * 4
        out = np.einsum('dij,deab->eiajb', out, w).reshape(dims[k + 1], out.shape[1] * 2, out.shape[2] * 2)
    return out[0]


def _dense_from_terms(n, terms):
    P = {'I': np.eye(2), 'X': np.array([[0, 1], [1, 0]]), 'Y': np.array([[0, -1j], [1j, 0]]),
         'Z': np.diag([1, -1])}
    H = np.zeros((2 ** n, 2 ** n), dtype=np.complex128)
    for c, ops in terms:
        m = np.ones((1, 1))
        for q in range(n):
            p = ops.get(q, 'I')
            p = {0: 'I', 1: 'X', 2: 'Y', 3: 'Z'}.get(p, p)
            m = np.kron(m, P[p])
        H += c * m
    return H


def test_pauli_mpo_equals_the_dense_sum():
    n = 5
    terms = AD.ising_terms(n, hx=0.3) + [(0.7, {0: 'Y', 3: 'X'}), (-1.1, {1: 3, 2: 1, 4: 2}), (0.25, {4: 'Z'})]
    dims, W = AD.pauli_mpo(n, terms)
    assert dims[0] == 1 and dims[-1] == 1
    np.testing.assert_allclose(_dense_from_mpo(n, dims, W), _dense_from_terms(n, terms), atol=1e-14)


def test_pauli_mpo_rejects_constants_and_out_of_range():
    with pytest.raises(ValueError):
        AD.pauli_mpo(3, [(1.0, {0: 'I'})])
    with pytest.raises(ValueError):
        AD.pauli_mpo(3, [(1.0, {3: 'Z'})])


def test_gradient_workload_builders_match_the_oracle():
    ang = OA.ansatz_angles(4, 2, seed=2)
    p = {'ry': torch.tensor(1e-3, dtype=torch.float64), 'rz': torch.tensor(2e-3, dtype=torch.float64),
         'cz': torch.tensor(1e-2, dtype=torch.float64)}
    mine = AD.hea_ops(ang, p)
    ref = OA.ansatz_ops(ang, p)
    assert len(mine) == len(ref)
    for a, b in zip(mine, ref):
        assert a[0] == b[0]
        if a[0] == '1q':
            assert a[1] == b[1]
            torch.testing.assert_close(a[2], b[2], rtol=0, atol=1e-15)
        elif a[0] == '2q':
            assert (a[1], a[1] + 1) == (b[1], b[2])
            torch.testing.assert_close(a[2], b[3], rtol=0, atol=1e-15)
    torch.testing.assert_close(AD.depolarization(torch.tensor(0.01, dtype=torch.float64), 2), O.depolarization(0.01, 2), rtol=0,
                               atol=1e-15)
