"""The GPU adjoint (mpdo_program_grad through mpdo_gb300.adjoint): loss and
gradients of the hardware-efficient ansatz (RY / RZ sublayers and a CZ
ladder, one trainable depolarising probability per gate type, Ising energy
sum Z_i Z_{i+1} + 0.5 sum X_i) against the gradient oracle (torch autograd
through the oracle's evolution, oracle/adjoint.py) and against central finite
differences of the GPU loss itself, with chi and kappa binding; and per-Kraus
gradients of a noisy brickwork (2q gates fused into the QR sweep, wide QR
factors at the chain ends) against autograd through the oracle."""
import math

import numpy as np
import pytest
import torch

from oracle import adjoint as OA, mpdo_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def AD():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    from mpdo_gb300 import adjoint
    return adjoint


def _params(n, layers, seed):
    ang = OA.ansatz_angles(n, layers, seed=seed)
    p = {k: torch.tensor(v, dtype=torch.float64) for k, v in (('ry', 2e-2), ('rz', 1e-2), ('cz', 3e-2))}
    return ang, p


def _oracle_energy(ang, p, chi, kappa):
    """oracle/adjoint.py's energy with the split's absolute cutoff off: the
    engine materialises 2q gates by QR and never drops the tail under the
    reference's cutoff (Circuit.py:116-126, a tail of norm up to
    sqrt(2 |theta| 2.7e-8) under its norm-difference rule)."""
    n = ang.shape[2]
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, OA.ansatz_ops(ang, p), chi=chi, kappa=kappa, noisy=True, cutoff=0.0)
    return OA.ising_energy(st)


def _gpu_energy(AD, ang, p, chi, kappa, dtype):
    n = ang.shape[2]
    return AD.program_loss(AD.hea_ops(ang, p), n, AD.ising_terms(n), chi, kappa, dtype=dtype)


@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-7), ('complex64', 3e-3)])
def test_ansatz_gradient_matches_oracle_autograd(AD, dtype, tol):
    n, layers, chi, kappa = 5, 2, 4, 2
    ang, p = _params(n, layers, seed=3)
    a1 = ang.clone().requires_grad_(True)
    p1 = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    e_ref = _oracle_energy(a1, p1, chi, kappa)
    e_ref.backward()
    a2 = ang.clone().requires_grad_(True)
    p2 = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    e = _gpu_energy(AD, a2, p2, chi, kappa, dtype)
    e.backward()
    print(f'\n{dtype}: energy {e.item():.10f} oracle {e_ref.item():.10f}; '
          f'max |dE/dangle - oracle| {(a2.grad - a1.grad).abs().max().item():.2e} '
          f'(max |dE/dangle| {a1.grad.abs().max().item():.2e})')
    assert abs(e.item() - e_ref.item()) < max(tol, 1e-9) * max(1.0, abs(e_ref.item()))
    scale = a1.grad.abs().max().item()
    assert (a2.grad - a1.grad).abs().max().item() <= tol * scale
    for k in p:
        assert abs(p2[k].grad.item() - p1[k].grad.item()) <= tol * max(abs(p1[k].grad.item()), scale)


def test_ansatz_gradient_matches_central_differences(AD):
    # complex128 central differences (h = 1e-4) of the GPU loss itself
    n, layers, chi, kappa = 5, 2, 4, 2
    ang, p = _params(n, layers, seed=4)
    a = ang.clone().requires_grad_(True)
    e = _gpu_energy(AD, a, p, chi, kappa, 'complex128')
    e.backward()
    h = 1e-4
    for idx in [(0, 0, 0), (0, 1, 2), (1, 0, 4), (1, 1, 1)]:
        ap, am = ang.clone(), ang.clone()
        ap[idx] += h
        am[idx] -= h
        fd = (_gpu_energy(AD, ap, p, chi, kappa, 'complex128').item()
              - _gpu_energy(AD, am, p, chi, kappa, 'complex128').item()) / (2 * h)
        assert abs(a.grad[idx].item() - fd) < 1e-7 + 1e-6 * abs(fd), (idx, a.grad[idx].item(), fd)


def _brickwork_ops(n, layers, seed):
    rng = np.random.default_rng(seed)
    dep1, dep2, dec = O.depolarization(0.02), O.depolarization(0.05, 2), O.amplitude_damping(0.03)
    ops = []
    for L in range(layers):
        for q in range(n):
            ops.append(('1q', q, O.noisy_1q(dec, dep1, O.gate_1q('U3', *(rng.random(3) * 2 * math.pi)))))
        ops.append(('truncate',))
        for q in range(L % 2, n - 1, 2):
            ops.append(('2q', q, q + 1, O.noisy_2q(dep2, O.gate_2q('CZ' if rng.random() < 0.5 else 'CNOT'))))
        ops.append(('truncate',))
    return ops


def test_brickwork_kraus_gradients_match_oracle_autograd(AD):
    n, layers, chi, kappa = 6, 3, 6, 3
    ops = _brickwork_ops(n, layers, seed=9)
    terms = AD.ising_terms(n)
    # oracle: autograd through the evolution with every Kraus tensor a leaf
    leaves = [op[-1].clone().requires_grad_(True) if op[0] != 'truncate' else None for op in ops]
    oops = [op[:-1] + (leaf,) if leaf is not None else op for op, leaf in zip(ops, leaves)]
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, oops, chi=chi, kappa=kappa, noisy=True, cutoff=0.0)
    Z, X = torch.as_tensor(O._PAULI[3]), torch.as_tensor(O._PAULI[1])
    e_ref = sum(O.expect_ops(st, {i: Z, i + 1: Z}) for i in range(n - 1)) + \
        0.5 * sum(O.expect_ops(st, {i: X}) for i in range(n))
    e_ref.backward()
    # GPU adjoint on the same Kraus tensors (2q legs in (min, max) order)
    gops = []
    for op in ops:
        if op[0] == '1q':
            gops.append(('1q', op[1], op[2]))
        elif op[0] == '2q':
            gops.append(('2q', min(op[1], op[2]), O.orient_2q(op[1], op[2], op[3])[1]))
        else:
            gops.append(op)
    loss, grads = AD.program_grad(gops, n, terms, chi, kappa, dtype='complex128')
    assert abs(loss - e_ref.item()) < 1e-8
    worst = 0.0
    scale = max(l.grad.abs().max().item() for l in leaves if l is not None)
    for leaf, g in zip(leaves, grads):
        if leaf is None:
            continue
        worst = max(worst, float(np.abs(g.reshape(leaf.shape) - leaf.grad.numpy()).max()))
    print(f'\nbrickwork n={n}: loss {loss:.10f}, max |dL/dK - oracle| {worst:.2e} (scale {scale:.2e})')
    # The oracle splits each 2q gate by SVD and keeps the numerical rank there;
    # the engine fuses the gate into the QR sweep and truncates at the next
    # SVD sweep.  The two functions agree at the evaluation point; their
    # derivatives differ in directions that populate exactly-zero singular
    # directions of a split (the split drops them, the fused path keeps them
    # until the sweep): a few 1e-5 of the gradient scale here.
    assert worst <= 1e-4 * scale
    # the engine's gradient is the derivative of the engine's own loss:
    # central differences (h = 1e-5) on entries of a 1q and a 2q Kraus tensor
    h = 1e-5
    for j in (0, next(i for i, op in enumerate(gops) if op[0] == '2q')):
        t = np.asarray(gops[j][2], dtype=np.complex128)
        for idx in [(0, 0, 0), (1, 0, 1)] if t.ndim == 3 else [(0, 0, 0, 0, 0), (1, 1, 0, 1, 3)]:
            for ph in (1, 1j):
                tp, tm = t.copy(), t.copy()
                tp[idx] += h * ph
                tm[idx] -= h * ph
                lp = AD.program_grad(gops[:j] + [(gops[j][0], gops[j][1], tp)] + gops[j + 1:], n, terms, chi, kappa,
                                     dtype='complex128')[0]
                lm = AD.program_grad(gops[:j] + [(gops[j][0], gops[j][1], tm)] + gops[j + 1:], n, terms, chi, kappa,
                                     dtype='complex128')[0]
                fd = (lp - lm) / (2 * h)
                g = grads[j][idx]
                an = g.real if ph == 1 else g.imag
                assert abs(an - fd) <= 1e-6 * scale, (j, idx, ph, an, fd)
