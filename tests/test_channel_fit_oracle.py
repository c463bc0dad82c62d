"""CPU pins of the channel-fitting checker (oracle/channel_fit.py): the
hidden channel is CPTP, the Choi-matrix proxy behaves as a distance, the
fit loss's gradient through the realNoise 2q path matches central finite
differences, and a short Adam run lowers the loss."""
import math

import torch

from oracle import channel_fit as C

N, DEPTH, CHI, KAPPA = 4, 3, 16, 4


def _loss(W, circs, data):
    K = C.kraus(C.stiefel(W))
    return sum(((C.marginals(a, K, CHI, KAPPA) - d) ** 2).sum() for a, d in zip(circs, data))


def test_hidden_channel_is_cptp_and_near_identity():
    V = C.hidden_isometry(7, 0.05)
    torch.testing.assert_close(V.conj().T @ V, torch.eye(4, dtype=V.dtype), rtol=0, atol=1e-14)
    K = C.kraus(V)
    J = C.choi(K)
    assert abs(torch.trace(J).real.item() - 1) < 1e-14
    assert torch.linalg.eigvalsh(J).min().item() > -1e-14
    ident = torch.zeros(4, 4, 4, dtype=torch.complex128)
    ident[0] = torch.eye(4)
    assert C.diamond_proxy(K, K) < 1e-14
    assert 0.01 < C.diamond_proxy(ident, K) < 0.5


def test_fit_loss_gradient_matches_central_fd():
    K_true = C.kraus(C.hidden_isometry(7, 0.05))
    circs = [C.random_circuit(N, DEPTH, s) for s in range(2)]
    data = [C.marginals(a, K_true, CHI, KAPPA) for a in circs]
    W0 = C.hidden_isometry(1, 1e-2)
    W = W0.clone().requires_grad_(True)
    _loss(W, circs, data).backward()
    h = 1e-6
    for idx in [(0, 0), (1, 2), (5, 1), (12, 3)]:
        for ph in (1, 1j):
            wp, wm = W0.clone(), W0.clone()
            wp[idx] += h * ph
            wm[idx] -= h * ph
            with torch.no_grad():
                fd = (float(_loss(wp, circs, data)) - float(_loss(wm, circs, data))) / (2 * h)
            ad = W.grad[idx].real.item() if ph == 1 else W.grad[idx].imag.item()
            assert abs(ad - fd) < 1e-6 * max(1.0, abs(fd)), (idx, ph, ad, fd)


def test_short_fit_lowers_the_loss():
    K_true = C.kraus(C.hidden_isometry(7, 0.05))
    circs = [C.random_circuit(N, DEPTH, s) for s in range(4)]
    data = [C.marginals(a, K_true, CHI, KAPPA) for a in circs]
    h = C.fit(circs, data, CHI, KAPPA, steps=8, lr=0.02, K_true=K_true)
    assert all(map(math.isfinite, h['loss'])) and h['loss'][-1] < h['loss'][0] / 5
    assert all(0 <= p < 1 for p in h['proxy'])


def test_identity_start_is_stationary_for_dissipative_directions():
    # at the exact identity channel the three zero Kraus operators enter rho
    # quadratically: their gradient vanishes (the bonds there are rank
    # deficient, which the gradient oracle handles by keeping the numerical rank)
    K_true = C.kraus(C.hidden_isometry(7, 0.05))
    circs = [C.random_circuit(N, DEPTH, s) for s in range(2)]
    data = [C.marginals(a, K_true, CHI, KAPPA) for a in circs]
    W = C.hidden_isometry(1, 0.0).clone().requires_grad_(True)
    _loss(W, circs, data).backward()
    assert torch.isfinite(W.grad).all()
    assert W.grad[:4].abs().max() > 1e-3 and W.grad[4:].abs().max() < 1e-12
