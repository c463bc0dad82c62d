"""Channel fitting on the GPU (mpdo_gb300.channel_fit): marginals and the
fit loss's gradient with respect to the Stiefel parameter W against the CPU
checker (oracle/channel_fit.py, torch autograd through the oracle's
evolution), and a short Adam run that lowers the loss."""
import numpy as np
import pytest
import torch

from oracle import channel_fit as C

pytestmark = pytest.mark.gpu

N, DEPTH, CHI, KAPPA = 4, 3, 16, 4


@pytest.fixture(scope='module')
def F():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    from mpdo_gb300 import channel_fit
    return channel_fit


def test_builders_match_the_checker(F):
    torch.testing.assert_close(F.hidden_isometry(7, 0.05), C.hidden_isometry(7, 0.05), rtol=0, atol=1e-14)
    K = F.kraus(F.hidden_isometry(7, 0.05))
    torch.testing.assert_close(F.cz_channel_tensor(K), C.cz_channel_tensor(K), rtol=0, atol=1e-14)
    torch.testing.assert_close(F.random_angles(N, DEPTH, 3), C.random_circuit(N, DEPTH, 3), rtol=0, atol=0)


@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-4), ('complex64', 2e-3)])
def test_marginals_and_gradient_match_the_checker(F, dtype, tol):
    K_true = C.kraus(C.hidden_isometry(7, 0.05))
    circs = [C.random_circuit(N, DEPTH, s) for s in range(2)]
    data = torch.stack([C.marginals(a, K_true, CHI, KAPPA) for a in circs])
    W0 = C.hidden_isometry(1, 1e-2)
    W1 = W0.clone().requires_grad_(True)
    K1 = C.kraus(C.stiefel(W1))
    ref = torch.stack([C.marginals(a, K1, CHI, KAPPA) for a in circs])
    ((ref - data) ** 2).sum().backward()
    fitter = F.Fitter(circs, CHI, KAPPA, dtype=dtype, workers=2)
    W2 = W0.clone().requires_grad_(True)
    m = fitter.marginals(F.cz_channel_tensor(F.kraus(F.stiefel(W2))))
    ((m - data) ** 2).sum().backward()
    err_m = (m.detach() - ref.detach()).abs().max().item()
    err_g = (W2.grad - W1.grad).abs().max().item()
    scale = W1.grad.abs().max().item()
    print(f'\n{dtype}: marginals {err_m:.2e}, dloss/dW {err_g:.2e} (scale {scale:.2e})')
    # marginals: the checker splits each CZ by SVD with the reference's cutoff,
    # the engine fuses it into the QR sweep (tail weight ~1e-8 apart).  The
    # gradient: the checker keeps the numerical rank at that split, the
    # engine carries the exactly-zero directions to the next sweep, so the
    # derivatives differ in directions that populate those zeros (4e-5 of
    # the gradient scale; the engine's own central differences agree,
    # tests/test_adjoint_gpu.py)
    assert err_m < (2e-7 if dtype == 'complex128' else 1e-5)
    assert err_g <= tol * scale


def test_short_fit_lowers_the_loss(F):
    K_true = C.kraus(C.hidden_isometry(7, 0.05))
    circs = [C.random_circuit(N, DEPTH, s) for s in range(4)]
    fitter = F.Fitter(circs, CHI, KAPPA, dtype='complex128', workers=4)
    data = fitter.marginals(F.cz_channel_tensor(K_true)).detach()
    hist = F.fit(fitter, data, steps=8, lr=0.02, K_true=K_true)
    print('\nloss', [f'{x:.2e}' for x in hist['loss']], 'proxy', [f'{x:.3f}' for x in hist['proxy']])
    assert hist['loss'][-1] < hist['loss'][0] / 5
