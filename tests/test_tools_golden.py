"""The drop-in host utilities (MPDOSimulator/Tools.py) against outputs of the
reference's own Tools module on the same seeded inputs
(tests/golden/tools.json, made by tests/golden/make_tools_golden.py)."""
import json
import os
import sys

import numpy as np
import pytest
import torch

import golden_io as G

sys.path.insert(0, G.GOLDEN)
from make_tools_golden import inputs  # noqa: E402

with open(os.path.join(G.GOLDEN, 'tools.json')) as _f:
    REF = json.load(_f)


def _arr(d):
    return (np.asarray(d['re']) + 1j * np.asarray(d['im'])).reshape(d['shape'])


@pytest.fixture(scope='module')
def T():
    from MPDOSimulator import Tools
    return Tools


@pytest.fixture(scope='module')
def x():
    return inputs()


def _close_dict(a, b, tol=1e-13):
    assert list(a.keys()) == list(b.keys())
    for k in a:
        assert abs(a[k] - b[k]) < tol, k


def test_density2prob(T, x):
    _close_dict(T.density2prob(x['rho']), REF['density2prob'])
    _close_dict(T.density2prob(x['rho'], tol=0.1), REF['density2prob_tol'])
    np.testing.assert_allclose(T.density2prob(x['rho'], _dict=False), REF['density2prob_array'], atol=1e-13)
    _close_dict(T.density2prob(x['rho'], bases=x['bases']), REF['density2prob_bases'])


def test_tc_expect(T, x):
    c = torch.complex128
    Z, X = T.name2matrix('ZII', dtype=c), T.name2matrix('IXI', dtype=c)
    np.testing.assert_allclose(T.tc_expect(Z, x['rho']).numpy(), _arr(REF['tc_expect_dm']), atol=1e-13)
    np.testing.assert_allclose(T.tc_expect(X, x['psi']).numpy(), _arr(REF['tc_expect_ket']), atol=1e-13)
    np.testing.assert_allclose(T.tc_expect([Z, X], x['rho']).numpy(), _arr(REF['tc_expect_list']), atol=1e-13)


def test_sqrt_matrix_and_fidelity(T, x):
    np.testing.assert_allclose(T.sqrt_matrix(x['rho']).numpy(), _arr(REF['sqrt_matrix']), atol=1e-12)
    np.testing.assert_allclose(T.sqrt_matrix(x['pure']).numpy(), _arr(REF['sqrt_matrix_pure']), atol=1e-12)
    assert abs(float(T.cal_fidelity(x['rho'], x['sigma']).real) - REF['cal_fidelity']) < 1e-12
    assert abs(float(T.cal_fidelity(x['rho'], x['rho']).real) - REF['cal_fidelity_self']) < 1e-12
    assert abs(float(T.cal_fidelity(x['pure'], x['rho']).real) - REF['cal_fidelity_pure']) < 1e-12


def test_matrices_lists_and_counts(T):
    c = torch.complex128
    np.testing.assert_array_equal(T.name2matrix('XYZ', dtype=c).numpy(), _arr(REF['name2matrix_XYZ']))
    assert T.gates_list(2) == REF['gates_list_2']
    assert T.gates_list(2, ['X', 'Z']) == REF['gates_list_xz']
    assert [[list(k), v] for k, v in T.count_item([[0, 1], [1, 0], [0, 1], [1, 1]]).items()] == \
        REF['count_item_lists']
    assert [[k, v] for k, v in T.count_item(['011', '100', '011', '001']).items()] == REF['count_item_strings']
    assert [[list(map(bool, k)), v] for k, v in
            T.count_item([[True, False], [False, False], [True, False]]).items()] == REF['count_item_bools']
    for name in ('ket_plus', 'ket_minus', 'ket_hadamard', 'ket1'):
        np.testing.assert_array_equal(getattr(T, name)(c).numpy(), _arr(REF[name]))
