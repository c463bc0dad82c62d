"""Batched evolution (mpdo_batch_run / MPDOSimulator.evolve_batch): every
circuit of a batch must end exactly as when evolved alone, whatever worker
ran it and whatever ran beside it; failures stay with their circuit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mods():
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    import mpdo_gb300
    mpdo_gb300.build()
    import MPDOSimulator as S
    from mpdo_gb300.workloads import build_circuit, u3_brickwork
    return S, build_circuit, u3_brickwork


def _circuits(S, build_circuit, u3_brickwork, specs):
    out = []
    for n, depth, chi, kappa, seed, dt in specs:
        w = u3_brickwork(n=n, depth=depth, chi=chi, kappa=kappa, seed=seed)
        out.append(build_circuit(w, dtype=dt, device='cuda:0'))
    return out


SPECS = [(6, 3, 8, 2, 0, torch.complex128), (8, 4, 16, 4, 1, torch.complex64), (5, 2, 4, 2, 2, torch.complex128),
         (10, 3, 16, 2, 3, torch.complex64), (7, 5, 8, 4, 4, torch.complex64), (6, 2, 32, 4, 5, torch.complex128)]


def test_evolve_batch_equals_single_evolve(mods):
    S, build_circuit, u3_brickwork = mods
    single = _circuits(S, build_circuit, u3_brickwork, SPECS)
    batched = _circuits(S, build_circuit, u3_brickwork, SPECS)
    for c in single:
        c.evolve(S.Tools.create_ket0Series(c.qnumber, dtype=c.dtype, connected=True))
    states = [S.Tools.create_ket0Series(c.qnumber, dtype=c.dtype, connected=True) for c in batched]
    res = S.evolve_batch(batched, states, workers=4)
    assert len({r['worker'] for r in res}) > 1
    for a, b, r in zip(single, batched, res):
        tol = 1e-12 if a.dtype == torch.complex128 else 1e-6
        da, db = a.cal_dm([0, 1]).cpu().numpy(), b.cal_dm([0, 1]).cpu().numpy()
        assert np.abs(da - db).max() <= tol
        assert len(a.discarded_weights) == len(b.discarded_weights)
        for x, y in zip(a.discarded_weights, b.discarded_weights):
            np.testing.assert_allclose(x, y, rtol=1e-6, atol=1e-12)
        n = a.qnumber
        z_ref = [S.dmOperations.pauli_expect(a.cal_dmNodes(), [2], [i]) for i in range(n)]
        np.testing.assert_allclose(r['z'], np.array([float(z) for z in z_ref]), atol=tol * 10)
        assert b.stateNodes[0].tensor.shape == a.stateNodes[0].tensor.shape


def test_batch_runs_many_circuits_on_few_workers(mods):
    S, build_circuit, u3_brickwork = mods
    specs = [(6, 2, 8, 2, s, torch.complex64) for s in range(12)]
    cs = _circuits(S, build_circuit, u3_brickwork, specs)
    ref = _circuits(S, build_circuit, u3_brickwork, specs)
    res = S.evolve_batch(cs, [S.Tools.create_ket0Series(6, dtype=torch.complex64, connected=True) for _ in cs],
                         workers=3)
    for c, r in zip(ref, res):
        c.evolve(S.Tools.create_ket0Series(6, dtype=torch.complex64, connected=True))
        zz_ref = [float(S.dmOperations.pauli_expect(c.cal_dmNodes(), [2, 2], [i, i + 1])) for i in range(5)]
        np.testing.assert_allclose(r['zz'], zz_ref, atol=1e-5)


def test_batch_failure_stays_with_its_circuit(mods):
    from mpdo_gb300 import Batch
    S, build_circuit, u3_brickwork = mods
    good = dict(n=4, dtype='complex64', vectors=[[1, 0]] * 4, connected=True, chi=4, kappa=2, noisy=True,
                ops=[('1q', 0, np.eye(2)[:, :, None]), ('2q', 1, np.eye(4).reshape(2, 2, 2, 2)), ('truncate',)],
                z=True)
    bad = dict(good, ops=[('1q', 7, np.eye(2)[:, :, None])])
    b = Batch.get(0, 2)
    with pytest.raises(ValueError, match='circuit 1'):
        b.run([good, bad, good])
    res = b.run([good, good])
    np.testing.assert_allclose(res[0]['z'], [1, 1, 1, 1], atol=1e-6)
