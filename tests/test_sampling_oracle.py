"""The conditional probabilities that drive sampling (Circuit.py:297-332)
against the reference's own, on the CPU: the oracle replays each golden
circuit's gate tensors, applies the measurement basis changes of the
orientation (MeasureX / MeasureY, Circuit.py:413-418) and must return the
reference's p(1 | prefix) for every prefix of length 0..2
(tests/golden/sampling.json, made by tests/golden/make_sampling_golden.py)."""
import json
import os
import sys

import pytest
import torch

import golden_io as G
from oracle import mpdo_oracle as O

sys.path.insert(0, G.GOLDEN)
from make_sampling_golden import CIRCUITS  # noqa: E402

with open(os.path.join(G.GOLDEN, 'sampling.json')) as _f:
    REF = json.load(_f)


@pytest.mark.parametrize('name', CIRCUITS)
def test_conditional_probabilities_match_reference(name):
    info, ops, _ = G.load(name)
    n = info['qn']
    st0 = O.product_state([[1, 0]] * n, connected=False, dtype=G.dtype_of(info))
    O.evolve(st0, ops, chi=info['chi'], kappa=info['kappa'], max_err=info['max_truncation_err'],
             noisy=not info['ideal'], randomized=info['randomized_svd_calls'] > 0)
    # where the reference took its randomized SVD branch (decompositions.py:112-115)
    # its state carries that branch's approximation error (4.3e-6 on rho); the
    # ratios p(1 | prefix) show it as ~2.6e-5
    tol = 5e-5 if info['randomized_svd_calls'] else 1e-10
    tables = [k for k in REF if k.startswith(name + ':')]
    assert len(tables) == 2
    for key in tables:
        orient = REF[key]['orientation']
        st = st0.clone()
        for q, v in enumerate(orient):
            if v in (0, 1):
                O.apply_1q(st, q, O.gate_1q('MEASUREX' if v == 0 else 'MEASUREY', dtype=torch.complex64)
                           .to(torch.complex128))
        order = list(range(n))
        for prefix, p1 in REF[key]['p1'].items():
            got = O.conditional_p1(st, order, [int(b) for b in prefix])
            assert abs(got - p1) <= tol, (key, prefix, got, p1)
