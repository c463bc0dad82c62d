"""The drop-in dmOperations host logic (DMNodes bookkeeping, traced qubits,
overlaps and composite purities; MPDOSimulator/dmOperations.py) against the
reference's own dmOperations on the same evolved states
(tests/golden/dmops.json, made by tests/golden/make_dmops_golden.py).

The engine chain behind DMNodes is replaced, in this test only, by a
stand-in that answers its two readout calls (reduced_dm, expect_ops) from
the oracle replaying the golden circuits' gate tensors; the GPU engine's
own readouts are checked against the oracle in the GPU tests."""
import json
import os
import sys

import numpy as np
import pytest
import torch

import golden_io as G
from oracle import mpdo_oracle as O

sys.path.insert(0, G.GOLDEN)
from make_dmops_golden import PAIR, TRACED  # noqa: E402

with open(os.path.join(G.GOLDEN, 'dmops.json')) as _f:
    REF = json.load(_f)


class _OracleChain:
    """Test stand-in for the engine chain's readout calls."""

    def __init__(self, st):
        self.st, self.n = st, st.n

    def reduced_dm(self, keep):
        return O.reduced_dm(self.st, keep).numpy()

    def expect_ops(self, ops):
        return float(O.expect_ops(self.st, {q: torch.as_tensor(o) for q, o in ops.items()}))


def _state(name):
    info, ops, _ = G.load(name)
    st = O.product_state([[1, 0]] * info['qn'], connected=False, dtype=G.dtype_of(info))
    O.evolve(st, ops, chi=info['chi'], kappa=info['kappa'], max_err=info['max_truncation_err'],
             noisy=not info['ideal'])
    return st


@pytest.mark.parametrize('tag', ['full', 'reduced'])
def test_dm_operations_match_reference(tag):
    from MPDOSimulator import dmOperations as D
    chains = [_OracleChain(_state(name)) for name in PAIR]
    n = chains[0].n

    def nodes(ch):
        d = D.DMNodes(ch, n, torch.complex128, 'cpu')
        if tag == 'reduced':
            D.reduce_dmNodes(d, reduced_index=TRACED)
        return d

    a, b = nodes(chains[0]), nodes(chains[1])
    ref = REF[tag]
    got = {'trace_rho': float(D.trace_rho(a)), 'trace_rho2': float(D.trace_rho2(a)),
           'trace_rho_rho': float(D.trace_rho_rho(a, b)),
           'trace_composited_rho': float(D.trace_composited_rho(a, b)),
           'trace_composited_rho2': float(D.trace_composited_rho2(a, b))}
    for k, v in ref.items():
        assert abs(got[k] - v) < 1e-10, (k, got[k], v)


def test_cal_vector_and_reduced_dm_host_logic():
    # TensorCircuit.cal_vector (Circuit.py:264-272) contracts the site tensors
    # read back from the chain on the host; cal_dm(reduced_index) maps traced
    # qubits to the kept list.  The noiseless golden circuit is pure, so the
    # reference's rho is |psi><psi|.
    import MPDOSimulator as S
    info, _, dm_ref = G.load('ideal_chi_c128')
    n = info['qn']

    class Chain(_OracleChain):
        def site(self, k):
            return self.st.sites[k].numpy()

    c = S.TensorCircuit(n, ideal=True, dtype=torch.complex128, device='cpu')
    c._chain = Chain(_state('ideal_chi_c128'))
    psi = c.cal_vector().numpy()[:, 0]
    assert np.abs(np.outer(psi, psi.conj()) - dm_ref).max() < 1e-10
    t = dm_ref.reshape([2] * (2 * n))
    for q in (2, 0):                                   # trace qubits 2 and 0 out of the reference's rho
        t = np.trace(t, axis1=q, axis2=q + t.ndim // 2)
    want = t.reshape(2 ** (n - 2), 2 ** (n - 2))
    assert np.abs(c.cal_dm([0, 2]).numpy() - want).max() < 1e-10
