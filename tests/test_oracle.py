"""CPU checks of the oracle: physics pins against the dense simulator and
analytic known answers (no GPU)."""

import numpy as np
import pytest
import torch

from oracle import mpdo_oracle as O, dense_dm as D
from circuits import brickwork


def test_no_truncation_equals_dense():
    n = 3
    ops = brickwork(n, 2, seed=3)
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, ops, chi=8, kappa=8, noisy=True)
    np.testing.assert_allclose(O.reduced_dm(st).numpy(), D.run(n, ops).numpy(), atol=1e-12)


def test_depolarizing_known_answer():
    # NoiseChannel.py:69-71: rho -> (1-p) rho + p I/2
    p = 0.3
    st = O.product_state([[1, 0]])
    O.apply_1q(st, 0, O.depolarization(p))
    rho = O.reduced_dm(st).numpy()
    np.testing.assert_allclose(rho, (1 - p) * np.diag([1, 0]) + p * np.eye(2) / 2, atol=1e-14)
    t = O.depolarization(p, 2)
    assert t.shape == (2, 2, 2, 2, 16)
    # completeness: sum_k K^dag K = I
    k = t.reshape(4, 4, 16)
    np.testing.assert_allclose(torch.einsum('abk,ack->bc', k.conj(), k).numpy(), np.eye(4), atol=1e-14)


@pytest.mark.parametrize('chan', ['ad', 'deph', 'apde'])
def test_channels_trace_preserving(chan):
    t = {'ad': O.amplitude_damping(0.2), 'deph': O.dephasing(0.01, 0.98, 30),
         'apde': O.amp_phase_damping(30, 2e2, 2e1)}[chan]
    np.testing.assert_allclose(torch.einsum('abk,ack->bc', t.conj(), t).numpy(), np.eye(2), atol=1e-14)


def test_ghz_known_answer():
    n = 5
    ops = [('1q', 0, O.gate_1q('H'))] + [('2q', q, q + 1, O.gate_2q('CNOT')) for q in range(n - 1)]
    st = O.product_state([[1, 0]] * n)
    O.evolve(st, ops + [('truncate',)], chi=4)
    p = O.density2prob(O.reduced_dm(st))
    assert abs(p[0] - 0.5) < 1e-12 and abs(p[-1] - 0.5) < 1e-12
    # parity <X...X> = 1
    assert abs(O.pauli_expect(st, [0] * n, list(range(n))).item() - 1) < 1e-12


def test_trace_preserved_without_truncation():
    n = 4
    ops = brickwork(n, 1, seed=9)
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, ops, chi=16, kappa=16, noisy=True)          # neither cap binds on this circuit
    assert abs(O.trace(st) - 1) < 1e-12


def test_gauge_invariance():
    # a unitary on a Kraus leg or on a bond leaves rho unchanged
    n = 4
    ops = brickwork(n, 2, seed=4)
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, ops, chi=6, kappa=3, noisy=True)
    rho = O.reduced_dm(st)
    g = torch.Generator().manual_seed(0)
    a = st.sites[1].shape[2]
    u, _ = torch.linalg.qr(torch.randn(a, a, dtype=torch.complex128, generator=g))
    st.sites[1] = torch.einsum('lsar,ab->lsbr', st.sites[1], u)
    b = st.sites[2].shape[3]
    v, _ = torch.linalg.qr(torch.randn(b, b, dtype=torch.complex128, generator=g))
    st.sites[2] = torch.einsum('lsar,rq->lsaq', st.sites[2], v)
    st.sites[3] = torch.einsum('qr,rsac->qsac', v.conj().T, st.sites[3])
    np.testing.assert_allclose(O.reduced_dm(st).numpy(), rho.numpy(), atol=1e-13)


def test_truncation_rule():
    # decompositions.py:121-132: keep idx+1 at the first idx with
    # ||s|| - ||s[:idx+1]|| <= err (difference of norms, not norm of the rest)
    s = torch.tensor([1.0, 0.1, 1e-4, 1e-9], dtype=torch.float64)
    m = torch.diag(s).to(torch.complex128)
    _, kept, _, rest = O.svd_truncate(m, None, 1e-7)
    assert kept.numel() == 2          # ||s|| - ||s[:2]|| ~ 5e-9 <= 1e-7
    _, kept, _, _ = O.svd_truncate(m, 3, 1e-12)
    assert kept.numel() == 3
    _, kept, _, _ = O.svd_truncate(m, None, 1e-2, relative=True)
    assert kept.numel() == 1


def test_disconnected_truncate_is_skipped():
    st = O.product_state([[1, 0]] * 3)
    O.apply_1q(st, 0, O.noisy_1q(O.amplitude_damping(0.1), O.depolarization(0.1), O.gate_1q('H')))
    before = st.dims()
    O.truncate(st, 2, 1, None, noisy=True)
    assert st.dims() == before


def test_reduced_dm_matches_partial_trace():
    n = 4
    ops = brickwork(n, 1, seed=2)
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, ops, chi=16, kappa=16, noisy=True)
    full = O.reduced_dm(st).numpy().reshape([2] * 8)
    red = np.einsum('abcdAbCd->acAC', full).reshape(4, 4)     # keep qubits 0, 2
    np.testing.assert_allclose(O.reduced_dm(st, [0, 2]).numpy(), red, atol=1e-13)


def test_chi_to_kraus_reproduces_ideal_cz():
    # a rank-1 process matrix of CZ in the (-iY) Pauli basis gives one Kraus op = CZ (up to phase)
    import itertools
    names = [''.join(g) for g in itertools.product('IXYZ', repeat=2)]
    cz = np.diag([1, 1, 1, -1]).astype(np.complex128)
    basis = [O._name2matrix(nm) for nm in names]
    c = np.array([np.trace(b.conj().T @ cz) / 4 for b in basis])  # cz = sum c_j P_j (P_j orthogonal, norm 4)
    chi = np.outer(c, c.conj())
    t = O.chi_to_kraus(chi)
    assert t.shape == (2, 2, 2, 2, 1)
    k = t[..., 0].reshape(4, 4).numpy()
    ph = k[0, 0] / abs(k[0, 0])
    np.testing.assert_allclose(k / ph, cz, atol=1e-12)


def test_expect_dense_against_the_dense_simulator():
    # dmOperations.py:135-171: Tr(rho_oq . O) for a two-qubit observable given
    # on qubits listed out of order (no truncation binds: rho is exact)
    n = 3
    ops = brickwork(n, 2, seed=21)
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, ops, chi=8, kappa=8, noisy=True)
    rho = D.run(n, ops)
    g = torch.Generator().manual_seed(3)
    a = torch.complex(torch.randn(4, 4, dtype=torch.float64, generator=g),
                      torch.randn(4, 4, dtype=torch.float64, generator=g))
    obs = (a + a.conj().T).reshape(2, 2, 2, 2)            # [out q2, out q0, in q2, in q0]
    eye = torch.eye(2, dtype=torch.complex128)
    full = torch.einsum('xyuv,pq->ypxvqu', obs, eye).reshape(8, 8)   # rows (s0, s1, s2), columns (t0, t1, t2)
    want = torch.trace(rho @ full).real.item()
    assert abs(O.expect_dense(st, obs.reshape(4, 4), [2, 0]).item() - want) < 1e-12
