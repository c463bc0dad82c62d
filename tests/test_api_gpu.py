"""The drop-in MPDOSimulator API on the GPU: config-0 workload, known answers,
readout functions and sampling."""
import math

import numpy as np
import pytest
import torch

from oracle import mpdo_oracle as O, dense_dm as D

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def S():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    import MPDOSimulator
    return MPDOSimulator


def _oracle_ops(w):
    dec = O.amplitude_damping(w.noise['gamma'])
    dep = O.depolarization(w.noise['p1'])
    dp2 = O.depolarization(w.noise['p2'], 2)
    ops = []
    for L in w.layers:
        if L[0] == '1q':
            ops.append(('1q', L[3], O.noisy_1q(dec, dep, O.gate_1q(L[1], *L[2]))))
        elif L[0] == '2q':
            ops.append(('2q', L[3], L[4], O.noisy_2q(dp2, O.gate_2q(L[1], *L[2]))))
        else:
            ops.append(('truncate',))
    return ops


@pytest.fixture(scope='module')
def brickwork_oracle():
    from mpdo_gb300.workloads import ry_rz_cnot_brickwork
    w = ry_rz_cnot_brickwork()
    ops = _oracle_ops(w)
    st = O.product_state([[1, 0]] * w.n, connected=True)
    O.evolve(st, ops, chi=w.chi, kappa=w.kappa, noisy=True)
    return w, ops, O.reduced_dm(st).numpy()


@pytest.mark.parametrize('dtype,tol', [(torch.complex128, 1e-6), (torch.complex64, 1e-5)])
def test_small_brickwork_matches_oracle(S, brickwork_oracle, dtype, tol):
    # the n=8, 8-layer RY/RZ/CNOT brickwork (chi=16, kappa=4): full 256x256 rho and the Z-basis
    # probabilities.  complex128 differs from the oracle only by the split cutoff
    # the fused path skips (tail weight ~1e-8); complex64 within 1e-5.
    from mpdo_gb300.workloads import build_circuit
    w, ops, ref = brickwork_oracle
    c = build_circuit(w, dtype=dtype, device='cuda:0')
    c.evolve(S.Tools.create_ket0Series(w.n, dtype=dtype, connected=True))
    rho = c.cal_dm().cpu().numpy()
    assert rho.shape == (256, 256)
    assert np.abs(rho - ref).max() < tol
    p = S.Tools.density2prob(torch.as_tensor(rho), _dict=False)
    assert np.abs(p - O.density2prob(torch.as_tensor(ref))).max() < tol
    # discarded weight is reported per truncate layer and per bond
    assert len(c.discarded_weights) == w.gate_layers
    # truncation error against the exact dense simulation is physical, not numerical
    exact = D.run(w.n, ops).numpy()
    assert np.abs(rho - exact).max() < 0.05


def test_ghz_ideal(S):
    n = 6
    c = S.TensorCircuit(n, ideal=True, chi=4, dtype=torch.complex128, device='cuda:0')
    c.h(0)
    for q in range(n - 1):
        c.cnot(q, q + 1)
    c.truncate()
    c.evolve(S.Tools.create_ket0Series(n, dtype=torch.complex128))
    v = c.cal_vector().cpu().numpy().ravel()
    ref = np.zeros(2 ** n, complex)
    ref[0] = ref[-1] = 1 / math.sqrt(2)
    assert abs(abs(np.vdot(ref, v)) - 1) < 1e-12
    dm = c.cal_dmNodes()
    assert abs(S.dmOperations.pauli_expect(dm, [0] * n, list(range(n))).item() - 1) < 1e-12
    samples, counts = c.sample(256, _tqdm_disable=True)
    assert set(counts) <= {'0' * n, '1' * n}


def test_depolarizing_known_answer(S):
    c = S.TensorCircuit(1, ideal=False, noiseType='idealNoise', dtype=torch.complex128, device='cuda:0')
    nz = c.Noise
    p = 0.2
    nz.dephasingTensor = nz.depolarization_noise_channel(p)
    nz.decayTensor = torch.as_tensor(np.stack([np.eye(2)], -1)).to(torch.complex128)
    c.i(0)
    c.evolve(S.Tools.create_ket0Series(1, dtype=torch.complex128))
    rho = c.cal_dm().cpu().numpy()
    np.testing.assert_allclose(rho, (1 - p) * np.diag([1, 0]) + p * np.eye(2) / 2, atol=1e-12)


def test_reduced_dm_expect_and_sampling(S):
    from mpdo_gb300.workloads import ry_rz_cnot_brickwork, build_circuit
    w = ry_rz_cnot_brickwork(n=5, depth=3, chi=8, kappa=4)
    ops = _oracle_ops(w)
    st = O.product_state([[1, 0]] * w.n, connected=True)
    O.evolve(st, ops, chi=w.chi, kappa=w.kappa, noisy=True, cutoff=0.0)
    c = build_circuit(w, dtype=torch.complex128, device='cuda:0')
    c.evolve(S.Tools.create_ket0Series(w.n, dtype=torch.complex128, connected=True))
    np.testing.assert_allclose(c.cal_dm(reduced_index=[0, 3]).cpu().numpy(), O.reduced_dm(st, [1, 2, 4]).numpy(),
                               atol=1e-10)
    dm = c.cal_dmNodes()
    z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex128)
    zz = torch.kron(z, z)
    e = S.dmOperations.expect(dm, [zz], [[3, 1]])[0].item()
    assert abs(e - O.expect_dense(st, zz, [3, 1]).item()) < 1e-10
    pe = S.dmOperations.pauli_expect(dm, [2, 0], [1, 4]).item()
    assert abs(pe - O.pauli_expect(st, [2, 0], [1, 4]).item()) < 1e-10
    assert abs(S.dmOperations.trace_rho(dm).item() - O.trace(st)) < 1e-10
    # sampling statistics against the Z-basis marginal of qubit 0
    torch.manual_seed(0)
    samples, counts = c.sample(4000, _tqdm_disable=True)
    p1 = sum(v for k, v in counts.items() if k[0] == '1') / 4000
    rho0 = O.reduced_dm(st, [0]).numpy()
    exact = rho0[1, 1].real / np.trace(rho0).real
    assert abs(p1 - exact) < 0.04
