"""GPU engine vs the CPU oracle through the C ABI (complex128 and complex64)."""
import numpy as np
import pytest
import torch

from oracle import mpdo_oracle as O, dense_dm as D
from circuits import brickwork, run_engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mg():
    mpdo_gb300 = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mpdo_gb300.build()
    return mpdo_gb300


def _oracle(n, ops, chi, kappa, dtype=torch.complex128, connected=True, noisy=True, max_err=None,
            cutoff=O.GLOBAL_MINIMUM):
    st = O.product_state([[1, 0]] * n, connected=connected, dtype=dtype)
    O.evolve(st, ops, chi=chi, kappa=kappa, max_err=max_err, noisy=noisy, cutoff=cutoff)
    return st


@pytest.fixture
def unfused(mg):
    eng = mg.Engine.get(0)
    eng.set_option('fuse_2q', 0)
    yield eng
    eng.set_option('fuse_2q', 1)


def test_apply_1q_matches_oracle(mg):
    rng = np.random.default_rng(1)
    ch = mg.Chain([[1, 0], [0.6, 0.8j]], dtype='complex128', connected=True)
    st = O.product_state([[1, 0], [0.6, 0.8j]], connected=True)
    k = rng.normal(size=(2, 2, 6)) + 1j * rng.normal(size=(2, 2, 6))
    ch.apply_1q(1, k)
    O.apply_1q(st, 1, torch.as_tensor(k))
    assert ch.site_dims(1) == tuple(st.sites[1].shape)
    np.testing.assert_allclose(ch.site(1), st.sites[1].numpy(), atol=1e-12)


def test_no_truncation_matches_dense(mg):
    n = 3
    ops = brickwork(n, 2, seed=3)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex128', connected=True), ops, chi=8, kappa=8)
    rho = ch.reduced_dm()
    rho_d = D.run(n, ops).numpy()
    assert abs(np.trace(rho) - 1) < 1e-10
    np.testing.assert_allclose(rho, rho_d, atol=1e-10)


CASES = [(4, 3, 4, 2), (6, 4, 8, 4), (5, 3, 6, 3)]


@pytest.mark.parametrize('n,layers,chi,kappa', CASES)
def test_truncated_c128_unfused_matches_oracle(mg, unfused, n, layers, chi, kappa):
    # the reference's exact sequence: SVD split with its cutoff, then the sweeps
    ops = brickwork(n, layers, seed=n + layers)
    st = _oracle(n, ops, chi, kappa)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex128', connected=True), ops, chi, kappa)
    assert ch.dims() == [tuple(s.shape) for s in st.sites]
    np.testing.assert_allclose(ch.reduced_dm(), O.reduced_dm(st).numpy(), atol=1e-10)


@pytest.mark.parametrize('n,layers,chi,kappa', CASES)
def test_truncated_c128_fused_matches_oracle(mg, n, layers, chi, kappa):
    # fused 2q + QR sweep == the reference sequence without the split cutoff;
    # the cutoff itself moves rho by its tail weight (~1e-8)
    ops = brickwork(n, layers, seed=n + layers)
    st0 = _oracle(n, ops, chi, kappa, cutoff=0.0)
    st = _oracle(n, ops, chi, kappa)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex128', connected=True), ops, chi, kappa)
    assert ch.dims() == [tuple(s.shape) for s in st.sites]
    rho_g = ch.reduced_dm()
    np.testing.assert_allclose(rho_g, O.reduced_dm(st0).numpy(), atol=1e-10)
    np.testing.assert_allclose(rho_g, O.reduced_dm(st).numpy(), atol=1e-6)


def test_truncated_c64_within_reference_sensitivity(mg):
    n, layers, chi, kappa = 6, 4, 8, 4
    ops = brickwork(n, layers, seed=7)
    st128 = _oracle(n, ops, chi, kappa)
    st64 = _oracle(n, [(o[0], *o[1:-1], o[-1].to(torch.complex64)) if o[0] in ('1q', '2q') else o for o in ops],
                   chi, kappa, dtype=torch.complex64)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex64', connected=True), ops, chi, kappa)
    r128 = O.reduced_dm(st128).numpy()
    intrinsic = np.abs(O.reduced_dm(st64).numpy().astype(np.complex128) - r128).max()
    err = np.abs(ch.reduced_dm() - r128).max()
    assert err <= max(1e-5, 4 * intrinsic), (err, intrinsic)


def test_materialized_split_matches_oracle(mg):
    # a 2q gate followed by readout (no truncate): the reference's SVD split
    n = 4
    ops = brickwork(n, 1, seed=11)
    ops = [o for o in ops if o[0] != 'truncate']
    st = _oracle(n, ops, None, None, noisy=False)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex128', connected=True), ops, None, None, noisy=False)
    np.testing.assert_allclose(ch.reduced_dm(), O.reduced_dm(st).numpy(), atol=1e-10)
    assert ch.dims() == [tuple(s.shape) for s in st.sites]


def test_disconnected_start_skips_truncate(mg):
    n = 3
    ops = brickwork(n, 1, seed=5)
    st = _oracle(n, ops, 4, 2, connected=False)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex128', connected=False), ops, 4, 2)
    assert ch.dims() == [tuple(s.shape) for s in st.sites]
    np.testing.assert_allclose(ch.reduced_dm(), O.reduced_dm(st).numpy(), atol=1e-10)


def test_readouts(mg):
    n = 5
    ops = brickwork(n, 2, seed=2)
    st = _oracle(n, ops, 6, 3)
    ch = run_engine(mg.Chain([[1, 0]] * n, dtype='complex128', connected=True), ops, 6, 3)
    for keep in ([0], [1, 3], [2, 3, 4]):
        np.testing.assert_allclose(ch.reduced_dm(keep), O.reduced_dm(st, keep).numpy(), atol=1e-10)
    p = ch.probs()
    np.testing.assert_allclose(p, np.diagonal(O.reduced_dm(st).numpy()).real, atol=1e-10)
    codes = np.zeros((3, n), dtype=np.int8)
    codes[0, 0] = 3
    codes[1, 1] = 3; codes[1, 2] = 3
    codes[2, 4] = 1
    vals = ch.expect_pauli_batch(codes)
    ref = [O.pauli_expect(st, [2], [0]).item(), O.pauli_expect(st, [2, 2], [1, 2]).item(),
           O.pauli_expect(st, [0], [4]).item()]
    np.testing.assert_allclose(vals, ref, atol=1e-10)
