"""Site tensors crossing the C ABI in device memory
(mpdo_chain_read_site_device / mpdo_chain_write_site_device): the same
values as the host copies, without a host round trip, and host pointers
rejected before any copy."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mg():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    return mg


SHAPES = [(1, 2, 2, 3), (3, 2, 1, 2), (2, 2, 3, 1)]      # consistent bonds of a 3-site chain


def _sites(seed):
    rng = np.random.default_rng(seed)
    return [rng.normal(size=s) + 1j * rng.normal(size=s) for s in SHAPES]


@pytest.mark.parametrize('dtype', ['complex64', 'complex128'])
def test_device_copies_equal_host_copies(mg, dtype):
    tdt = torch.complex64 if dtype == 'complex64' else torch.complex128
    sites = _sites(5)
    via_dev = mg.Chain([[1, 0]] * 3, dtype=dtype, connected=True)
    via_host = mg.Chain([[1, 0]] * 3, dtype=dtype, connected=True)
    for k, a in enumerate(sites):
        t = torch.tensor(a, dtype=tdt, device='cuda:0')
        via_dev.write_site_tensor(k, t)
        via_host.write_site(k, t.cpu().numpy())
    for k, a in enumerate(sites):
        want = torch.tensor(a, dtype=tdt)
        got = via_dev.site_tensor(k)
        assert got.device.type == 'cuda' and got.dtype == tdt and tuple(got.shape) == SHAPES[k]
        assert torch.equal(got.cpu(), want)                              # bit-exact round trip
        assert np.array_equal(via_dev.site(k), want.numpy().astype(np.complex128))
        assert torch.equal(via_host.site_tensor(k).cpu(), want)         # host write, device read
    np.testing.assert_array_equal(via_dev.reduced_dm([0, 1, 2]), via_host.reduced_dm([0, 1, 2]))
    # a CPU tensor given to write_site_tensor is brought to the engine's device first
    via_dev.write_site_tensor(1, torch.tensor(sites[1], dtype=torch.complex128))
    assert torch.equal(via_dev.site_tensor(1).cpu(), torch.tensor(sites[1], dtype=tdt))


def test_host_pointer_is_rejected(mg):
    from mpdo_gb300 import _lib
    ch = mg.Chain([[1, 0]] * 2, dtype='complex64', connected=True)
    host = np.zeros(64, dtype=np.complex64)
    lib = _lib.load()
    st = lib.mpdo_chain_read_site_device(ch.handle, 0, C.c_void_p(host.ctypes.data))
    assert st == _lib.MPDO_ERR_INVALID and b'device memory' in lib.mpdo_last_error()
    dims = (C.c_int * 4)(1, 2, 1, 1)
    st = lib.mpdo_chain_write_site_device(ch.handle, 0, dims, C.c_void_p(host.ctypes.data))
    assert st == _lib.MPDO_ERR_INVALID
    assert np.array_equal(ch.site(0), np.array([1, 0], dtype=np.complex128).reshape(1, 2, 1, 1))   # unchanged


def test_drop_in_state_nodes_read_from_device(mg):
    import MPDOSimulator as S
    from mpdo_gb300.workloads import build_circuit, ry_rz_cnot_brickwork
    w = ry_rz_cnot_brickwork(n=5, depth=2)
    c = build_circuit(w, dtype=torch.complex64, device='cuda:0')
    c.evolve(S.Tools.create_ket0Series(w.n, dtype=torch.complex64, connected=True))
    ch = c._need_chain()
    for k, node in enumerate(c.stateNodes):
        t = node.tensor
        assert t.device.type == 'cuda' and t.dtype == torch.complex64
        assert np.array_equal(t.cpu().numpy().astype(np.complex128), ch.site(k))
