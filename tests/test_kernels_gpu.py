"""Kernel-level GPU tests through the C-ABI test hooks: Householder QR (incl.
TSQR levels) and QR + one-sided Jacobi SVD against numpy.  The complex64
tolerances sit 3-10x above the errors measured on a GB300 for these seeded
inputs (QR 2.6e-7, right SVD 3.8e-6, split 1.3e-6, wide splits 4e-9 to
3.2e-6, tridiagonal route 5.4e-7), on the scales each assertion states."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def eng():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    return mg.Engine.get(0)


def _rand(m, n, seed, rank=None):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
    if rank is not None:
        u, s, vh = np.linalg.svd(a, full_matrices=False)
        s[rank:] = 0
        a = (u * s) @ vh
    return a


@pytest.mark.parametrize('m,n', [(8, 8), (40, 13), (13, 40), (512, 64), (4096, 64), (33000, 32), (300, 150)])
@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-11), ('complex64', 1e-6)])
def test_qr(eng, m, n, dtype, tol):
    a = _rand(m, n, m + n)
    q, r = eng.debug_qr(a, dtype)
    k = min(m, n)
    assert np.abs(q @ r - a).max() <= tol * np.abs(a).max() * 4
    assert np.abs(q.conj().T @ q - np.eye(k)).max() <= tol * 10
    assert np.abs(np.tril(r, -1)).max() == 0


@pytest.mark.parametrize('m,n,rank', [(64, 64, None), (100, 20, None), (20, 100, None), (64, 64, 10), (256, 48, 5),
                                      (16, 3, 1)])
@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-10), ('complex64', 1e-5)])
def test_right_svd(eng, m, n, rank, dtype, tol):
    a = _rand(m, n, 7 * m + n, rank)
    w, s = eng.debug_svd(a, dtype)
    s_ref = np.linalg.svd(a, compute_uv=False)
    k = min(m, n)
    np.testing.assert_allclose(s[:k], s_ref[:k], atol=tol * s_ref[0])
    assert np.all(np.diff(s) <= 1e-12 * s[0] + tol * s[0])          # sorted descending
    assert np.abs(w.conj().T @ w - np.eye(n)).max() <= tol * 10        # unitary even when rank deficient
    # A W has orthogonal columns with norms s
    aw = a @ w
    g = aw.conj().T @ aw
    np.testing.assert_allclose(np.sqrt(np.abs(np.diag(g))), s, atol=tol * 10 * s_ref[0])
    off = g - np.diag(np.diag(g))
    assert np.abs(off).max() <= tol * 10 * s_ref[0] ** 2


@pytest.mark.parametrize('m,n,keep,rank', [(8, 512, 8, None), (32, 1024, 8, None), (8, 1024, 8, 3), (64, 16, 8, None),
                                           (16, 4, 10, None), (256, 8192, 64, None), (4, 200, 6, None)])
@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-10), ('complex64', 5e-6)])
def test_split(eng, m, n, keep, rank, dtype, tol):
    y = _rand(m, n, 3 * m + n, rank)
    L, R = eng.debug_split(y, keep, dtype)
    u, s, vh = np.linalg.svd(y, full_matrices=False)
    k = min(keep, len(s))
    best = (u[:, :k] * s[:k]) @ vh[:k]
    np.testing.assert_allclose(L @ R, best, atol=tol * s[0] * 10)
    # L = U sqrt(S): orthogonal columns with squared norms = s
    g = L.conj().T @ L
    np.testing.assert_allclose(np.diag(g).real[:k], s[:k], rtol=tol * 10, atol=tol * s[0])
    if keep > k:
        assert np.abs(L[:, k:]).max() == 0 and np.abs(R[k:]).max() == 0


@pytest.mark.parametrize('dtype,scale,tol', [('complex128', 1e-160, 1e-11), ('complex64', 1e-21, 1e-6)])
def test_qr_columns_near_underflow(eng, dtype, scale, tol):
    # rank-deficient factors carry junk directions whose squares underflow;
    # the reflectors must stay unitary (scaled norms)
    a = _rand(128, 64, 5)
    a[:, 40:] *= scale
    a[60:, 48:] = 0
    q, r = eng.debug_qr(a, dtype)
    assert np.isfinite(q).all() and np.isfinite(r).all()
    assert np.abs(q.conj().T @ q - np.eye(64)).max() <= tol * 10
    assert np.abs(q @ r - a).max() <= tol * np.abs(a).max() * 4
    w, s = eng.debug_svd(a, dtype)
    assert np.isfinite(w).all() and np.abs(w.conj().T @ w - np.eye(64)).max() <= tol * 10


@pytest.mark.parametrize('m,n,keep,rank', [(128, 2048, 128, 20), (256, 8192, 64, 40), (200, 300, 150, 7)])
@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-10), ('complex64', 1e-6)])
def test_split_wide_rank_deficient(eng, m, n, keep, rank, dtype, tol):
    # wide bonds go through the Gram / block-Jacobi / Rayleigh-Ritz path; exact
    # rank deficiency must not break the orthonormality of the basis
    y = _rand(m, n, 11 * m + n, rank)
    L, R = eng.debug_split(y, keep, dtype)
    u, s, vh = np.linalg.svd(y, full_matrices=False)
    k = min(keep, len(s))
    best = (u[:, :k] * s[:k]) @ vh[:k]
    np.testing.assert_allclose(L @ R, best, atol=tol * s[0] * 10)


def _decaying(m, n, seed, decades_per_sv):
    rng = np.random.default_rng(seed)
    u, _ = np.linalg.qr(rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m)))
    v, _ = np.linalg.qr(rng.normal(size=(n, m)) + 1j * rng.normal(size=(n, m)))
    s = 10.0 ** (-np.arange(m) * decades_per_sv)
    return (u * s) @ v.conj().T


@pytest.mark.parametrize('decay,expect_range', [(0.25, True), (0.01, False)])
@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-10), ('complex64', 1e-5)])
def test_split_wide_range_finder(eng, decay, expect_range, dtype, tol):
    # wide bonds first try the randomized range finder; it is accepted only when
    # the residual outside its span is at rounding level (fast-decaying
    # spectrum), otherwise the exact block-Jacobi path runs.  Both must give the
    # best rank-keep approximation.
    m, n, keep = 256, 2048, 64
    y = _decaying(m, n, 21, decay)
    eng.profile(True)
    eng.set_option('wide_range', 1)
    try:
        L, R = eng.debug_split(y, keep, dtype)
    finally:
        eng.set_option('wide_range', -1)
    wide = eng.profile_read()['wide_bonds']
    eng.profile(False)
    assert (wide['range_finder'], wide['exact']) == ((1, 0) if expect_range else (0, 1))
    u, s, vh = np.linalg.svd(y, full_matrices=False)
    best = (u[:, :keep] * s[:keep]) @ vh[:keep]
    np.testing.assert_allclose(L @ R, best, atol=tol * s[0] * 10)
    g = L.conj().T @ L
    np.testing.assert_allclose(np.diag(g).real, s[:keep], atol=tol * s[0])
    assert np.abs(g - np.diag(np.diag(g))).max() <= tol * s[0]


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_split_wide_range_matches_exact(eng, dtype):
    # the same split through both wide paths (option wide_range on / off)
    y = _decaying(256, 4096, 5, 0.1)
    try:
        eng.set_option('wide_range', 1)
        L1, R1 = eng.debug_split(y, 64, dtype)
        eng.set_option('wide_range', 0)
        L0, R0 = eng.debug_split(y, 64, dtype)
    finally:
        eng.set_option('wide_range', -1)
    tol = 1e-11 if dtype == 'complex128' else 2e-5
    np.testing.assert_allclose(L1 @ R1, L0 @ R0, atol=tol * np.abs(L0 @ R0).max() * 10)


@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-10), ('complex64', 1e-6)])
def test_split_wide_512(eng, dtype, tol):
    # the pair bond at chi=128 (Mr = 512): Gram 512 x 512 through block Jacobi
    y = _decaying(512, 2048, 9, 0.02)
    L, R = eng.debug_split(y, 128, dtype)
    u, s, vh = np.linalg.svd(y, full_matrices=False)
    best = (u[:, :128] * s[:128]) @ vh[:128]
    np.testing.assert_allclose(L @ R, best, atol=tol * s[0] * 10)


@pytest.mark.parametrize('m,n,keep,decay', [(128, 1024, 64, 0.03), (200, 1500, 80, 0.02), (256, 2048, 64, 0.01),
                                            (256, 4096, 64, 0.003), (512, 2048, 128, 0.01)])
@pytest.mark.parametrize('dtype,tol', [('complex128', 1e-10), ('complex64', 3e-6)])
def test_split_wide_tridiagonal_matches_jacobi(eng, m, n, keep, decay, dtype, tol):
    # the exact wide path diagonalises the Gram by cluster tridiagonalisation
    # (default) or block Jacobi; both must give the best rank-keep approximation
    y = _decaying(m, n, m + keep, decay)
    u, s, vh = np.linalg.svd(y, full_matrices=False)
    best = (u[:, :keep] * s[:keep]) @ vh[:keep]
    eng.profile(True)
    try:
        eng.set_option('wide_range', 0)
        eng.set_option('wide_eig', 1)
        L1, R1 = eng.debug_split(y, keep, dtype)
        wide = eng.profile_read()['wide_bonds']
        eng.set_option('wide_eig', 0)
        L0, R0 = eng.debug_split(y, keep, dtype)
    finally:
        eng.set_option('wide_eig', -1)
        eng.set_option('wide_range', -1)
        eng.profile(False)
    # (the cluster holds up to 512 rows in complex64, 374 in complex128)
    assert wide['tridiagonal'] == (1 if m <= (512 if dtype == 'complex64' else 374) else 0)
    np.testing.assert_allclose(L1 @ R1, best, atol=tol * s[0] * 10)
    np.testing.assert_allclose(L0 @ R0, best, atol=tol * s[0] * 10)
    g = L1.conj().T @ L1
    np.testing.assert_allclose(np.diag(g).real, s[:keep], atol=tol * s[0])


@pytest.mark.parametrize('m,n,keep,bs', [(128, 2048, 64, 0), (256, 8192, 64, 0), (200, 600, 100, 0), (256, 4096, 64, 8)])
@pytest.mark.parametrize('dtype', ['complex64', 'complex128'])
def test_block_jacobi_cluster_matches_rounds(eng, m, n, keep, bs, dtype):
    # The wide-bond block Jacobi runs as one thread-block-cluster launch that
    # decides convergence on the device, or as one launch per tournament round
    # with the host reading the rotation flag after each sweep.  Same rounds,
    # same per-round arithmetic: the splits must agree to rounding (they are
    # identical on a GB300).  m=128 and 256 use 8-CTA clusters; m=200 has 17
    # blocks (a 9-CTA cluster) and m=256 with 8-column blocks a 16-CTA cluster,
    # both beyond the portable size of 8, which a GB300 accepts.
    y = _rand(m, n, 5 * m + n)
    out, launches = {}, {}
    eng.set_option('wide_eig', 0)      # block Jacobi in complex128 too
    eng.set_option('wide_range', 0)
    eng.set_option('bjacobi_bs', bs)
    try:
        for fused in (0, 1):
            eng.set_option('bjacobi_fused', fused)
            eng.profile(True)
            out[fused] = eng.debug_split(y, keep, dtype)
            launches[fused] = eng.profile_read()['bjacobi']['launches']
            eng.profile(False)
    finally:
        eng.set_option('bjacobi_fused', 1)
        eng.set_option('bjacobi_bs', 0)
        eng.set_option('wide_eig', -1)
        eng.set_option('wide_range', -1)
    (L0, R0), (L1, R1) = out[0], out[1]
    scale = np.abs(L0 @ R0).max()
    tol = 1e-12 if dtype == 'complex128' else 1e-6
    np.testing.assert_allclose(L1 @ R1, L0 @ R0, atol=tol * scale)
    np.testing.assert_allclose(np.abs(L1), np.abs(L0), atol=tol * np.abs(L0).max() * 10)
    assert launches[0] > 8                  # several outer sweeps of 15 or more rounds
    assert launches[1] == 1
    u, s, vh = np.linalg.svd(y, full_matrices=False)
    best = (u[:, :keep] * s[:keep]) @ vh[:keep]
    np.testing.assert_allclose(L1 @ R1, best, atol=(1e-10 if dtype == 'complex128' else 3e-5) * s[0] * 10)
