"""Tr(rho_0 rho_1) over many kept qubits (dmOperations.py:51-132).

CPU: the oracle's site-by-site contraction of the doubled network against
the product of dense reduced density matrices, and the drop-in's routing
beyond 12 kept qubits (diagonal plus twice the cross terms for composite
purities) on oracle-backed chains.  GPU: the engine's four-layer
environment sweep against the oracle, for kept and traced qubits, one state
and two, complex128 and complex64."""
import numpy as np
import pytest
import torch

from circuits import brickwork, run_engine
from oracle import mpdo_oracle as O


def _state(n, layers, seed, chi=8, kappa=2, dtype=torch.complex128):
    st = O.product_state([[1, 0]] * n, connected=True, dtype=dtype)
    O.evolve(st, brickwork(n, layers, seed=seed), chi=chi, kappa=kappa, noisy=True)
    return st


@pytest.mark.parametrize('keep', [[0, 1, 2, 3, 4, 5], [1, 2, 4], [0, 5], []])
def test_oracle_contraction_equals_dense(keep):
    a, b = _state(6, 2, 1), _state(6, 2, 2)
    got = O.trace_rho_rho(a, b, keep)
    ra, rb = O.reduced_dm(a, keep), O.reduced_dm(b, keep)
    ref = float(torch.trace(ra @ rb).real)
    assert abs(got - ref) < 1e-12 * max(1.0, abs(ref))
    assert abs(O.trace_rho_rho(a, a, keep) - float(torch.trace(ra @ ra).real)) < 1e-12


class _OracleChain:
    """Oracle-backed stand-in for the engine chain's readout calls."""

    def __init__(self, st):
        self.st, self.n, self.calls = st, st.n, []

    def trace_rho_rho(self, other, keep):
        self.calls.append(('trr', tuple(keep)))
        return O.trace_rho_rho(self.st, other.st, keep)

    def reduced_dm(self, keep):
        raise AssertionError('no dense reduced density matrix beyond 12 qubits')


def test_drop_in_beyond_twelve_qubits():
    from MPDOSimulator import dmOperations as D
    n = 14
    sts = [_state(n, 1, s, chi=4) for s in range(3)]
    nodes = []
    for st in sts:
        d = D.DMNodes(_OracleChain(st), n, torch.complex128, 'cpu')
        D.reduce_dmNodes(d, reduced_index=[5])
        nodes.append(d)
    keep = [q for q in range(n) if q != 5]
    assert abs(float(D.trace_rho_rho(nodes[0], nodes[1])) - O.trace_rho_rho(sts[0], sts[1], keep)) < 1e-14
    assert abs(float(D.trace_rho2(nodes[2])) - O.trace_rho_rho(sts[2], sts[2], keep)) < 1e-14
    tot = sum(O.trace_rho_rho(a, b, keep) for a in sts for b in sts) / 9
    assert abs(float(D.trace_composited_rho2(*nodes)) - tot) < 1e-14
    other = D.DMNodes(_OracleChain(sts[1]), n, torch.complex128, 'cpu')
    with pytest.raises(ValueError):
        D.trace_rho_rho(nodes[0], other)


@pytest.fixture(scope='module')
def mg():
    mpdo_gb300 = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mpdo_gb300.build()
    return mpdo_gb300


@pytest.mark.gpu
@pytest.mark.parametrize('dtype,tol,self_tol', [('complex128', 1e-9, 1e-12), ('complex64', 1e-4, 1e-5)])
def test_engine_sweep_matches_oracle(mg, dtype, tol, self_tol):
    # against the oracle's states: the engine fuses each 2q gate into the QR
    # sweep where the oracle splits it with the reference's cutoff, so the
    # states differ by that tail (1e-8 of weight at most); against the
    # engine's own reduced density matrices (up to 12 kept qubits) the sweep
    # must agree to rounding.  Tr(rho_i rho_k) is bilinear, so its error is
    # bounded on the scale sqrt(Tr rho_i^2 Tr rho_k^2) (Cauchy-Schwarz), not on
    # that of its value: the cross term of two different states is small
    # (1.6e-5 against purities near 1 here).  A purity is quadratic in rho, so
    # the complex64 state's 1e-5 error against the complex128 oracle shows
    # doubled there (tolerance 1e-4).
    n, chi, kappa = 14, 8, 2
    ops = [brickwork(n, 2, seed=s) for s in (3, 4)]
    sts = []
    chains = []
    for o in ops:
        st = O.product_state([[1, 0]] * n, connected=True)
        O.evolve(st, o, chi=chi, kappa=kappa, noisy=True)
        sts.append(st)
        ch = mg.Chain([[1, 0]] * n, dtype=dtype, connected=True)
        run_engine(ch, o, chi, kappa)
        chains.append(ch)
    for keep in (list(range(n)), [q for q in range(n) if q not in (0, 6, 13)], [1, 2, 3, 5, 8, 9, 12], [2, 9], []):
        pur = [float(O.trace_rho_rho(sts[j], sts[j], keep)) for j in (0, 1)]
        for i, k in ((0, 0), (0, 1), (1, 0)):
            scale = float(np.sqrt(pur[i] * pur[k]))
            got = chains[i].trace_rho_rho(chains[k], keep)
            ref = O.trace_rho_rho(sts[i], sts[k], keep)
            assert abs(got - ref) <= tol * scale, (keep, i, k, got, ref, scale)
            if len(keep) <= 12:
                r0, r1 = chains[i].reduced_dm(keep), chains[k].reduced_dm(keep)
                own = float(np.sum(r0 * r1.T).real)
                assert abs(got - own) <= self_tol * scale, (keep, i, k, got, own, scale)


@pytest.mark.gpu
def test_engine_sweep_through_the_drop_in(mg):
    import MPDOSimulator as S
    from mpdo_gb300.workloads import build_circuit, u3_brickwork
    w = u3_brickwork(n=13, depth=3, chi=8, kappa=2, seed=2)
    c = build_circuit(w, dtype=torch.complex128, device='cuda:0')
    c.evolve(S.Tools.create_ket0Series(13, dtype=torch.complex128, connected=True))
    d = c.cal_dmNodes()
    pur = float(S.dmOperations.trace_rho2(d))
    tr = float(S.dmOperations.trace_rho(d))
    # purity of the (unnormalised) noisy state: below Tr(rho)^2, positive
    assert 0 < pur < tr ** 2
    # against the reduced density matrices once two qubits are traced (11 kept)
    d2 = c.cal_dmNodes(reduced_index=[0, 12])
    rho = c._chain.reduced_dm(list(range(1, 12)))
    assert abs(float(S.dmOperations.trace_rho2(d2)) - float(np.sum(rho * rho.T).real)) < 1e-10
    assert abs(c._chain.trace_rho_rho(None, list(range(1, 12))) - float(np.sum(rho * rho.T).real)) < 1e-10
