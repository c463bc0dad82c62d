"""The drop-in API's host-side circuit building against the reference: the
golden fixtures hold the exact gate tensors the reference applied (composite
noisy 1q gates, Circuit.py:141-155; 2q gate with depolarising or the CZEXP
Kraus set of a chi matrix, Circuit.py:84-100 and RealNoise.py:22-179).  The
drop-in package builds the same circuits from the same API calls; every
applied operation must be the same quantum operation (compared as the
superoperator sum_k K_k (x) conj(K_k), which does not depend on the order or
phases of the Kraus operators)."""
import sys

import numpy as np
import pytest
import torch

import golden_io as G

sys.path.insert(0, G.GOLDEN)
from cases import CASES, HOST_CASES  # noqa: E402

ALL_CASES = {**CASES, **HOST_CASES}


def _drop_in_ops(c):
    """The (kind, qubits, tensor) sequence the drop-in's evolve applies."""
    ops = []
    for i, layer in enumerate(c.layers):
        name = layer.name.lower()
        if 'truncate' in name:
            ops.append(('truncate',))
            continue
        if 'barrier' in name or layer.name == 'MeasureZ':
            continue
        oqs = c._oqs_list[i]
        if layer.single:
            t = c._noisy_1q(layer)
            ops += [('1q', q, t) for q in oqs]
        else:
            ops.append(('2q', oqs[0], oqs[1], c._noisy_2q(layer)))
    return ops


def _superop(t, n_out):
    t = np.asarray(t, dtype=np.complex128)
    d = 2 ** n_out
    if t.ndim == 2 * n_out:
        t = t[..., None]
    k = t.reshape(d, d, -1)
    return np.einsum('ijk,lmk->iljm', k, k.conj()).reshape(d * d, d * d)


@pytest.mark.parametrize('name', sorted(ALL_CASES))
def test_drop_in_builds_reference_operations(name, tmp_path):
    import MPDOSimulator as S
    fn, dtype = ALL_CASES[name]
    c = fn(S, dtype, 'cpu', str(tmp_path))
    info, ref_ops, _ = G.load(name)
    mine = _drop_in_ops(c)
    assert [o[0] for o in mine] == [o[0] for o in ref_ops]
    tol = 1e-6 if dtype == torch.complex64 else 1e-12
    for j, (a, b) in enumerate(zip(mine, ref_ops)):
        if a[0] == 'truncate':
            continue
        nq = 1 if a[0] == '1q' else 2
        assert a[1:1 + nq] == b[1:1 + nq], f'op {j}: qubits {a[1:1 + nq]} != {b[1:1 + nq]}'
        sa, sb = _superop(a[-1], nq), _superop(b[-1].numpy(), nq)
        assert np.abs(sa - sb).max() <= tol, f'op {j} ({a[0]} on {a[1:1 + nq]}) differs'
