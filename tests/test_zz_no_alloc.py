"""Allocation-free SVD entry point (mpdo_right_svd_noalloc) against the
allocating one (mpdo_debug_svd), through the C ABI on the GPU.

The entry point serves callers that cannot allocate device memory (a process
whose device memory is pre-partitioned by its own allocator, or code under an
allocation hook): it works out of one fixed 8 MiB static device array.  This
file is collected last so that a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def env():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    from mpdo_gb300 import _lib
    return _lib.load(), mg.Engine.get(0)


def _noalloc(lib, a: np.ndarray):
    m, n = a.shape
    da = torch.as_tensor(a.astype(np.complex64)).cuda().contiguous()
    dw = torch.empty(n * n, dtype=torch.complex64, device='cuda')
    ds = torch.empty(n, dtype=torch.float32, device='cuda')
    dst = torch.full((1,), -1, dtype=torch.int32, device='cuda')
    torch.cuda.synchronize()
    st = lib.mpdo_right_svd_noalloc(m, n, C.c_void_p(da.data_ptr()), C.c_void_p(dw.data_ptr()),
                                    C.c_void_p(ds.data_ptr()), C.c_void_p(dst.data_ptr()), None)
    assert st == 0, lib.mpdo_last_error().decode()
    torch.cuda.synchronize()
    w = dw.cpu().numpy().reshape(n, n).T          # column-major on the device
    return w, ds.cpu().numpy(), int(dst.item())


def _check_against_allocating(eng, a, w, s):
    w_ref, s_ref = eng.debug_svd(a, 'complex64')
    tol = 2e-4
    np.testing.assert_allclose(s, s_ref, atol=tol * s_ref[0])
    # same algorithm on the same input: same vectors up to a phase per column
    k = int(np.sum(s_ref > 1e-3 * s_ref[0]))
    overlap = np.abs(np.sum(w[:, :k].conj() * w_ref[:, :k], axis=0))
    np.testing.assert_allclose(overlap, 1.0, atol=1e-3)
    np.testing.assert_allclose(w.conj().T @ w, np.eye(w.shape[0]), atol=tol * 10)


def test_noalloc_matches_allocating_entry_point_twice(env):
    lib, eng = env
    rng = np.random.default_rng(3)
    # two calls in a row with different inputs: the shared scratch keeps the
    # previous call's contents, which must not leak into the next result
    for m, n in ((4096, 64), (300, 17)):
        a = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
        w, s, status = _noalloc(lib, a)
        assert status == 0
        _check_against_allocating(eng, a, w, s)


def test_noalloc_rejects_oversized(env):
    lib, _ = env
    d = torch.empty(8, dtype=torch.complex64, device='cuda')
    st = lib.mpdo_right_svd_noalloc(100, 65, C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()),
                                    C.c_void_p(d.data_ptr()), None, None)
    assert st == 1 and b'outside the allocation-free limits' in lib.mpdo_last_error()
    st = lib.mpdo_right_svd_noalloc(8193, 8, C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()),
                                    C.c_void_p(d.data_ptr()), None, None)
    assert st == 1
