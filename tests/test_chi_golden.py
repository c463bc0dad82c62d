"""chi-matrix ingestion (RealNoise.py:22-179) against the reference's own
fixtures: the reference's chi/ideal_cz.mat and chi/czDefault.mat matrices
and the Kraus tensors the reference makes from them (tests/golden/chi.json,
made by tests/golden/make_chi_golden.py).  The oracle's chi_to_kraus and
the drop-in's RealNoise.czExp_channel must give the same quantum operation
(superoperator), and the ideal CZ process must give CZ itself."""
import json
import os

import numpy as np
import pytest
import torch

import golden_io as G
from oracle import mpdo_oracle as O

with open(os.path.join(G.GOLDEN, 'chi.json')) as _f:
    REF = json.load(_f)


def _arr(d):
    return (np.asarray(d['re']) + 1j * np.asarray(d['im'])).reshape(d['shape'])


def _superop(k):
    k = np.asarray(k, dtype=np.complex128).reshape(4, 4, -1)
    return np.einsum('ijk,lmk->iljm', k, k.conj()).reshape(16, 16)


@pytest.mark.parametrize('fn', ['ideal_cz.mat', 'czDefault.mat'])
def test_chi_to_kraus_matches_reference(fn, tmp_path):
    chi = _arr(REF[fn]['chi'])
    ref = _superop(_arr(REF[fn]['kraus']))
    # the reference builds its Kraus tensor in complex64 (RealNoise.py:164-170)
    tol = 1e-6 * max(1.0, np.abs(ref).max())
    assert np.abs(_superop(O.chi_to_kraus(chi).numpy()) - ref).max() < tol
    from MPDOSimulator import RealNoise
    path = str(tmp_path / 'chi.npz')
    np.savez(path, chi=chi)
    mine = RealNoise.czExp_channel(filename=path, dtype=torch.complex128).numpy()
    assert mine.shape == tuple(REF[fn]['kraus']['shape'])
    assert np.abs(_superop(mine) - ref).max() < tol


def test_ideal_cz_process_is_cz():
    k = _arr(REF['ideal_cz.mat']['kraus'])[..., 0].reshape(4, 4)
    ph = k[0, 0] / abs(k[0, 0])
    np.testing.assert_allclose(k / ph, np.diag([1, 1, 1, -1]), atol=1e-6)
