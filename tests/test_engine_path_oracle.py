"""The engine's order of operations (fused two-qubit gates, isometry
shortcut, zero padding; oracle/engine_path.py) against the reference path
(oracle/mpdo_oracle.py) on the CPU: the same state up to the split cutoff's
tail, and -- differentiated with the gradient oracle -- the same gradient,
which is what lets an adjoint differentiate the engine's own sequence."""
import numpy as np
import pytest
import torch

from circuits import brickwork
from oracle import adjoint as A, engine_path as E, mpdo_oracle as O


@pytest.mark.parametrize('n,depth,chi,kappa,seed', [(4, 2, 4, 2, 3), (5, 3, 4, 2, 4), (4, 3, 16, 4, 5)])
def test_engine_order_gives_the_reference_state(n, depth, chi, kappa, seed):
    ops = brickwork(n, depth, seed=seed)
    ref = O.evolve(O.product_state([[1, 0]] * n, connected=True), ops, chi=chi, kappa=kappa, noisy=True)
    eng = E.evolve(O.product_state([[1, 0]] * n, connected=True), ops, chi=chi, kappa=kappa, noisy=True)
    # the fused pairs skip the split's absolute cutoff (weight ~1e-8)
    assert np.abs(O.reduced_dm(ref).numpy() - O.reduced_dm(eng).numpy()).max() < 1e-7
    assert [s.shape[0] for s in eng.sites] == [s.shape[0] for s in ref.sites]


def test_engine_order_gives_the_reference_gradient():
    n, layers, chi, kappa = 5, 2, 4, 2
    ang = A.ansatz_angles(n, layers, seed=2)
    p = {k: torch.tensor(v, dtype=torch.float64) for k, v in (('ry', 1e-3), ('rz', 2e-3), ('cz', 1e-2))}
    out = []
    for path in (O.evolve, E.evolve):
        a1 = ang.clone().requires_grad_(True)
        p1 = {k: v.clone().requires_grad_(True) for k, v in p.items()}
        st = O.product_state([[1, 0]] * n, connected=True)
        path(st, A.ansatz_ops(a1, p1), chi=chi, kappa=kappa, noisy=True)
        e = A.ising_energy(st)
        e.backward()
        out.append((e.item(), a1.grad, [p1[k].grad.item() for k in p1]))
    (e0, g0, q0), (e1, g1, q1) = out
    assert abs(e0 - e1) < 1e-9
    torch.testing.assert_close(g1, g0, rtol=0, atol=1e-7)
    np.testing.assert_allclose(q1, q0, rtol=1e-7)
