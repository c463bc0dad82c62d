"""The standalone sweeps (TNNOptimizer.py:87-161: qr_left2right,
svd_right2left, svd_left2right) on the GPU against the oracle's
restatements, on random connected chains written into the engine site by
site: leg dimensions, the dense density matrix and the discarded weight per
bond; and the drop-in entry points on an evolved state."""
import numpy as np
import pytest
import torch

from oracle import mpdo_oracle as O

pytestmark = pytest.mark.gpu

TOL = {'complex128': 1e-11, 'complex64': 2e-5}


@pytest.fixture(scope='module')
def mg():
    mpdo_gb300 = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mpdo_gb300.build()
    return mpdo_gb300


def _random_chain(bonds, kraus, seed):
    g = np.random.default_rng(seed)
    sites = []
    for i, a in enumerate(kraus):
        shape = (bonds[i], 2, a, bonds[i + 1])
        sites.append(g.normal(size=shape) + 1j * g.normal(size=shape))
    return sites


def _both(mg, sites, dtype):
    n = len(sites)
    ch = mg.Chain([[1, 0]] * n, dtype=dtype, connected=True)
    for i, s in enumerate(sites):
        ch.write_site(i, s)
    tdt = torch.complex128 if dtype == 'complex128' else torch.complex64
    st = O.MPDO([torch.tensor(s, dtype=torch.complex128).to(tdt) for s in sites], [True] * (n - 1))
    return ch, st


def _rho_oracle(st):
    st64 = O.MPDO([s.to(torch.complex128) for s in st.sites], list(st.bonds))
    return O.reduced_dm(st64).numpy()


def _close(a, b, dtype):
    scale = np.abs(b).max()
    err = np.abs(a - b).max() / scale
    assert err < TOL[dtype], err


# bond dimensions wider than chi in both directions, Kraus legs 1..3
BONDS = [1, 4, 9, 12, 7, 3, 1]
KRAUS = [2, 1, 3, 2, 1, 2]


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_qr_left2right(mg, dtype):
    sites = _random_chain(BONDS, KRAUS, 1)
    ch, st = _both(mg, sites, dtype)
    rho0 = _rho_oracle(st)
    ch.qr_left2right()
    O.qr_left2right(st)
    assert ch.dims() == st.dims()
    _close(ch.reduced_dm(), rho0, dtype)
    for i in range(ch.n - 1):                              # left-orthonormal sites
        a = ch.site(i)
        m = a.reshape(-1, a.shape[-1])
        np.testing.assert_allclose(m.conj().T @ m, np.eye(m.shape[1]), atol=TOL[dtype] * 10)


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
@pytest.mark.parametrize('direction', ['right2left', 'left2right'])
@pytest.mark.parametrize('chi,max_err', [(3, None), (None, 5e-2), (5, 5e-2), (None, None)])
def test_svd_sweep(mg, dtype, direction, chi, max_err):
    sites = _random_chain(BONDS, KRAUS, 2)
    ch, st = _both(mg, sites, dtype)
    if direction == 'right2left':
        ch.qr_left2right()
        O.qr_left2right(st)
        disc_o = O.svd_right2left(st, chi, max_err)
    else:
        disc_o = O.svd_left2right(st, chi, max_err)
    disc = ch.svd_sweep(direction, chi, max_err)
    assert ch.dims() == st.dims()
    _close(ch.reduced_dm(), _rho_oracle(st), dtype)
    np.testing.assert_allclose(disc, disc_o, rtol=0, atol=1e-12 if dtype == 'complex128' else 1e-5)
    if chi is not None or max_err is not None:
        assert max(disc) > 0


def test_sweeps_need_a_connected_chain(mg):
    ch = mg.Chain([[1, 0]] * 3, dtype='complex128', connected=False)
    for f in (ch.qr_left2right, lambda: ch.svd_sweep('right2left', 2, None),
              lambda: ch.svd_sweep('left2right', 2, None)):
        with pytest.raises(Exception, match='share a bond'):
            f()


def test_drop_in_entry_points(mg):
    # evolve a small noisy circuit through the drop-in, then the reference's
    # sweep sequence bondTruncate = qr_left2right + svd_right2left by hand
    import MPDOSimulator as S
    from MPDOSimulator import TNNOptimizer as T
    # (kappa keeps the Kraus legs at 2: without it they grow 6-fold per layer)
    c = S.TensorCircuit(5, ideal=False, noiseType='unified', chi=None, kappa=2, dtype=torch.complex128,
                        device='cuda:0')
    for layer in range(4):
        for q in range(5):
            c.u3(0.3 + q + layer, 0.2 * q, -0.7, [q])
        for q in range(layer % 2, 4, 2):
            c.cz(q, q + 1) if layer % 3 else c.cnot(q, q + 1)
        c.truncate()
    nodes = c.evolve(S.Tools.create_ket0Series(5, dtype=torch.complex128, connected=True))
    ch = nodes[0]._chain
    rho = ch.reduced_dm()
    T.qr_left2right(nodes)
    _close(ch.reduced_dm(), rho, 'complex128')
    assert max(d[3] for d in ch.dims()) > 2
    disc = T.svd_right2left(nodes, 2)
    assert all(d[3] <= 2 for d in ch.dims()) and max(disc) > 0 and min(disc) >= 0
    T.svd_left2right(nodes, 2)
    assert all(d[3] <= 2 for d in ch.dims())
