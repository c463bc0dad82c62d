"""The drop-in gate library (MPDOSimulator/QuantumGates) against the
oracle's gate definitions (which cite QuantumGates/*.py of the reference),
on the CPU: every gate's matrix, its numpy fast path, and gradients flowing
through parameterised gates (the reference detaches them; the drop-in keeps
the angles differentiable)."""
import math

import numpy as np
import pytest
import torch

from oracle import mpdo_oracle as O

ONE = [('IGate', 'I', ()), ('HGate', 'H', ()), ('XGate', 'X', ()), ('YGate', 'Y', ()), ('ZGate', 'Z', ()),
       ('SGate', 'S', ()), ('SDGGate', 'SDG', ()), ('TGate', 'T', ()), ('RXGate', 'RX', (0.7,)),
       ('RYGate', 'RY', (1.3,)), ('RZGate', 'RZ', (-2.2,)), ('PGate', 'P', (0.4,)), ('U1Gate', 'U1', (2.5,)),
       ('U2Gate', 'U2', (0.3, -1.1)), ('U3Gate', 'U3', (0.9, 1.7, -0.6))]
TWO = [('CNOTGate', 'CNOT', ()), ('CXGate', 'CX', ()), ('CYGate', 'CY', ()), ('CZGate', 'CZ', ()),
       ('SWAPGate', 'SWAP', ()), ('ISWAPGate', 'ISWAP', ()), ('IIGate', 'II', ()), ('PSWAPGate', 'PSWAP', (0.8,)),
       ('CPGate', 'CP', (1.9,)), ('RXXGate', 'RXX', (0.5,)), ('RYYGate', 'RYY', (-1.2,)), ('RZZGate', 'RZZ', (2.1,)),
       ('XXPlusYYGate', 'XXPLUSYY', (0.6, 0.25))]


def _cls(name):
    from MPDOSimulator.QuantumGates import (DoubleGates, PhaseGates, SingleGates, XGates, YGates,  # noqa: F401
                                            ZGates)
    for mod in (SingleGates, XGates, YGates, ZGates, PhaseGates, DoubleGates):
        if hasattr(mod, name):
            return getattr(mod, name)
    raise AttributeError(name)


@pytest.mark.parametrize('cls,name,params', ONE)
def test_single_qubit_gates(cls, name, params):
    g = _cls(cls)(*params, dtype=torch.complex128)
    ref = O.gate_1q(name, *params).numpy()
    np.testing.assert_allclose(g.tensor.numpy(), ref, atol=1e-14)
    np.testing.assert_allclose(g.numpy_tensor() if hasattr(g, 'numpy_tensor') else g.tensor.numpy(), ref, atol=1e-14)


@pytest.mark.parametrize('cls,name,params', TWO)
def test_two_qubit_gates(cls, name, params):
    g = _cls(cls)(*params, dtype=torch.complex128)
    ref = O.gate_2q(name, *params).numpy().reshape(2, 2, 2, 2)
    np.testing.assert_allclose(g.tensor.numpy().reshape(2, 2, 2, 2), ref, atol=1e-14)
    np.testing.assert_allclose(g.numpy_tensor().reshape(2, 2, 2, 2), ref, atol=1e-14)


@pytest.mark.parametrize('cls', ['HGate', 'TGate', 'CNOTGate', 'ISWAPGate'])
@pytest.mark.parametrize('dtype', [torch.complex64, torch.complex128])
def test_fixed_gate_fast_path_holds_the_tensor_values(cls, dtype):
    # the host fast path carries the matrix entries rounded to the circuit
    # dtype, bit for bit what ``tensor`` holds
    g = _cls(cls)(dtype=dtype)
    t = g.tensor.to(torch.complex128).numpy()
    assert np.array_equal(g.numpy_tensor(), t)
    assert not g.numpy_tensor().flags.writeable


def test_number_angles_stay_on_the_host():
    # a gate for a CUDA device keeps angles given as numbers in host memory
    # (no device copy to build, none to read back for the engine); this runs
    # without CUDA
    g = _cls('U3Gate')(0.9, 1.7, -0.6, dtype=torch.complex64, device='cuda:0')
    assert all(p.device.type == 'cpu' and p.dtype == torch.float32 for p in g.para)
    ref = O.gate_1q('U3', *[float(torch.tensor(x, dtype=torch.float32)) for x in (0.9, 1.7, -0.6)]).numpy()
    np.testing.assert_allclose(g.numpy_tensor(), ref, atol=1e-15)


def test_gate_modules_behave_as_nn_modules():
    # gates create nn.Module's containers lazily; every module operation
    # must behave as after nn.Module.__init__, with containers per gate
    import copy
    import MPDOSimulator as S
    c = S.TensorCircuit(3, ideal=False, noiseType='unified', chi=4, kappa=2, device='cpu')
    c.u3(0.1, 0.2, 0.3, [0])
    c.cz(0, 1)
    c.rx(0.4, 2)
    c.truncate()
    g0, g1 = c.layers[0], c.layers[1]
    h = g0.register_forward_hook(lambda *a: None)
    assert len(g0._forward_hooks) == 1 and len(g1._forward_hooks) == 0
    h.remove()
    assert c.to('cpu') is c and c.state_dict() == {} and list(c.named_parameters()) == []
    c.eval()
    assert not g0.training
    c.train()
    assert g1.training
    assert len(list(c.modules())) == 6 and 'U3Gate()' in repr(c.layers)
    d = copy.deepcopy(c)
    assert abs(d.layers[0].para[0].item() - 0.1) < 1e-7 and d.layers[0] is not g0
    assert not hasattr(g1, '_build_np')
    with pytest.raises(AttributeError):
        g0.no_such_attribute
    g1.extra = torch.nn.Identity()                  # a submodule still registers
    assert 'extra' in dict(g1.named_children()) and len(list(c.modules())) == 7


def test_angles_stay_differentiable():
    th = torch.tensor(0.8, dtype=torch.float64, requires_grad=True)
    g = _cls('U3Gate')(th, 0.2, -0.4, dtype=torch.complex128)
    # the fast path must not be taken for a parameter that needs a gradient
    np.testing.assert_allclose(g.numpy_tensor(), g.tensor.detach().numpy(), atol=1e-15)
    loss = (g.tensor.abs() ** 2)[0, 0]                  # cos^2(theta / 2)
    loss.backward()
    assert abs(th.grad.item() + math.sin(0.8) / 2) < 1e-12


def test_workload_generators():
    from mpdo_gb300.workloads import u3_brickwork, uneven_batch_circuit
    w = u3_brickwork()
    assert (w.n, w.chi, w.kappa, w.gates, w.gate_layers) == (32, 64, 4, 950, 40)
    for s in range(16):
        c = uneven_batch_circuit(s)
        assert 12 <= c.n <= 40 and c.chi in (16, 32, 64, 128) and c.kappa in (2, 4)
        assert 10 <= c.depth <= 30 and c.gate_layers == 2 * c.depth
    assert uneven_batch_circuit(3).layers == uneven_batch_circuit(3).layers        # seeded


def test_engine_ops_follow_evolve_semantics():
    # Circuit.py:469-491: gate layers in order, one op per target of a 1q
    # layer, 2q tensors oriented (min, max), barriers and MeasureZ skipped,
    # a final kappa pass only when a noisy circuit does not end on truncate
    import MPDOSimulator as S
    c = S.TensorCircuit(3, ideal=False, noiseType='idealNoise', chi=4, kappa=2, dtype=torch.complex128,
                        device='cpu')
    c.h([0, 2])
    c.cnot(2, 1)
    c.barrier()
    c.truncate()
    c.measure([0])
    c.rz(0.3, [1])
    ops = c._engine_ops()
    kinds = [o[0] for o in ops]
    assert kinds == ['1q', '1q', '2q', 'truncate', '1q', 'kappa']
    assert ops[0][1] == 0 and ops[1][1] == 2 and ops[2][1] == 1
    assert ops[0][2].shape[:2] == (2, 2) and ops[2][2].shape[:4] == (2, 2, 2, 2)
    # CNOT with control 2 on the pair (1, 2): oriented to (min, max) legs
    t = ops[2][2]
    cnot = O.gate_2q('CNOT').numpy().reshape(2, 2, 2, 2)
    noisy = np.einsum('ijklp,klmn->ijmnp', np.asarray(c.Noise.dpCTensor2), cnot)    # Circuit.py:91-100
    np.testing.assert_allclose(t, np.transpose(noisy, (1, 0, 3, 2, 4)), atol=1e-12)
    ideal = S.TensorCircuit(2, ideal=True, dtype=torch.complex128, device='cpu')
    ideal.h([0])
    assert [o[0] for o in ideal._engine_ops()] == ['1q']


class _FakeChain:
    """Records the engine calls the TNNOptimizer entry points make."""

    def __init__(self, n, bonds=True):
        self.n, self.bonds, self.calls = n, bonds, []

    def bond_present(self, b):
        return self.bonds

    def truncate(self, *a):
        self.calls.append(('truncate',) + a)

    def kappa_truncate(self, *a):
        self.calls.append(('kappa',) + a)

    def qr_left2right(self):
        self.calls.append(('qr',))

    def svd_sweep(self, *a):
        self.calls.append(('svd',) + a)
        return [0.0] * (self.n - 1)


def test_tnnoptimizer_entry_points_map_to_engine_operations():
    # TNNOptimizer.py:51-197 on the nodes of an evolved state
    from MPDOSimulator import TNNOptimizer as T, Tools
    ch = _FakeChain(3)
    nodes = [Tools.QubitNode(None, f'qubit_{k}', [], chain=ch, index=k) for k in range(3)]
    assert T.bondTruncate(nodes) is None and T.svdKappa_left2right(nodes) is None and ch.calls == []
    T.bondTruncate(nodes, 8)
    T.bondTruncate(nodes, None, 1e-3)
    T.svdKappa_left2right(nodes, 4, 1e-3)
    assert ch.calls == [('truncate', 8, None, None, False), ('truncate', None, None, 1e-3, False),
                        ('kappa', 4, 1e-3)]
    assert T.checkConnectivity(nodes) and not T.checkConnectivity(
        [Tools.QubitNode(None, f'q{k}', [], chain=_FakeChain(2, bonds=False), index=k) for k in range(1)] * 2)
    assert not T.checkConnectivity(Tools.create_ket0Series(3)) and T.checkConnectivity(
        Tools.create_ket0Series(3, connected=True))
    with pytest.raises(TypeError):
        T.bondTruncate(tuple(nodes), 4)
    with pytest.raises(ValueError):
        T.bondTruncate(nodes[:2], 4)
    ch.calls.clear()
    T.qr_left2right(nodes)
    assert T.svd_right2left(nodes, 4) == [0.0, 0.0]
    T.svd_left2right(nodes, 2, 1e-6)
    assert ch.calls == [('qr',), ('svd', 'right2left', 4, None), ('svd', 'left2right', 2, 1e-6)]
    with pytest.raises(ValueError):
        T.svd_left2right(nodes[:1], 2)
