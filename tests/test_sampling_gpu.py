"""Conditional sampling on the GPU (Circuit.py:297-446 semantics): the
empirical distribution of many shots against the exact Z-basis (or rotated)
probabilities of the same state, deterministic states, traced qubits and
reproducibility under torch.manual_seed."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def S():
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    import MPDOSimulator
    return MPDOSimulator


def _noisy(S, n=6, depth=3, dtype=torch.complex128):
    from mpdo_gb300.workloads import u3_brickwork, build_circuit
    w = u3_brickwork(n=n, depth=depth, chi=8, kappa=2, seed=5)
    w.noise = dict(p1=0.02, gamma=0.03, p2=0.05)
    c = build_circuit(w, dtype=dtype, device='cuda:0')
    c.evolve(S.Tools.create_ket0Series(n, dtype=dtype, connected=True))
    return c


def _check_freq(bits, probs, shots):
    L = bits.shape[1]
    idx = bits.astype(np.int64) @ (1 << np.arange(L - 1, -1, -1))
    freq = np.bincount(idx, minlength=1 << L) / shots
    tol = 5 * np.sqrt(probs * (1 - probs) / shots) + 2e-3
    assert np.all(np.abs(freq - probs) <= tol), np.max(np.abs(freq - probs) - tol)


def test_deterministic_product_state(S):
    c = S.TensorCircuit(4, ideal=True, dtype=torch.complex64, device='cuda:0')
    c.x([1])
    c.x([3])
    c.evolve(S.Tools.create_ket0Series(4, dtype=torch.complex64))
    samples, counts = c.sample(500)
    assert counts == {'0101': 500}


def test_ghz_halves(S):
    c = S.TensorCircuit(5, ideal=True, dtype=torch.complex128, device='cuda:0')
    c.h([0])
    for q in range(4):
        c.cnot(q, q + 1)
    c.evolve(S.Tools.create_ket0Series(5, dtype=torch.complex128))
    torch.manual_seed(3)
    _, counts = c.sample(20000)
    assert set(counts) == {'00000', '11111'}
    assert abs(counts['11111'] / 20000 - 0.5) < 5 * np.sqrt(0.25 / 20000)


@pytest.mark.parametrize('dtype', [torch.complex128, torch.complex64])
def test_noisy_distribution_matches_probabilities(S, dtype):
    c = _noisy(S, dtype=dtype)
    p = c.probabilities().numpy()
    p = p / p.sum()
    shots = 40000
    torch.manual_seed(11)
    bits = np.array(c.sample(shots, sample_string=False, _require_counts=False))
    _check_freq(bits, p, shots)


def test_traced_qubits_and_rotated_basis(S):
    c = _noisy(S)
    # sample qubits 0, 1, 3, 4, 5 (qubit 2 traced) with X on the 2nd and Y on the 4th of them
    orient = [2, 0, 2, 1, 2]
    shots = 40000
    torch.manual_seed(7)
    bits = np.array(c.sample(shots, orientation=orient, reduced=[2], sample_string=False, _require_counts=False))
    ch = c._chain.clone()
    from MPDOSimulator.QuantumGates.SingleGates import MeasureX, MeasureY
    ch.apply_1q(1, c._np(MeasureX(dtype=c.dtype).tensor))
    ch.apply_1q(4, c._np(MeasureY(dtype=c.dtype).tensor))
    p = np.asarray(ch.probs([0, 1, 3, 4, 5]))
    _check_freq(bits, p / p.sum(), shots)


def test_reproducible_under_manual_seed(S):
    c = _noisy(S)
    torch.manual_seed(42)
    a = c.sample(3000, sample_string=False, _require_counts=False)
    torch.manual_seed(42)
    b = c.sample(3000, sample_string=False, _require_counts=False)
    assert a == b


def _loop_random_sample(c, schemes, shots, reduced):
    # Circuit.py:448-466 as the reference runs it: one sample() per scheme
    return [c.sample(shots, orientation=s, reduced=reduced, sample_string=False, _tqdm_disable=True,
                     _require_counts=False) for s in schemes]


@pytest.mark.parametrize('dtype', [torch.complex128, torch.complex64])
def test_random_sample_equals_the_per_scheme_loop(S, dtype):
    # one engine call for all schemes gives, scheme by scheme, the bits of the
    # reference's loop of sample() calls under the same torch seed
    c = _noisy(S, dtype=dtype)
    rng = np.random.default_rng(3)
    schemes = rng.integers(0, 3, size=(12, 5)).tolist() + [[2] * 5, [0] * 5, [1] * 5]
    torch.manual_seed(5)
    batched = c.randomSample(schemes, shots_per_scheme=2000, reduced=[2], _tqdm_disable=True)
    torch.manual_seed(5)
    loop = _loop_random_sample(c, schemes, 2000, [2])
    assert len(batched) == len(schemes)
    same = sum(a == b for a, b in zip(batched, loop))
    # complex64 probabilities may differ in the last bit between the two
    # orders of work, which moves a binomial draw in rare cases
    assert same == len(schemes) if dtype == torch.complex128 else same >= len(schemes) - 1


def test_random_sample_distributions(S):
    c = _noisy(S)
    schemes = [[0, 1, 2, 0, 1], [1, 1, 0, 2, 2]]
    shots = 40000
    torch.manual_seed(9)
    out = c.randomSample(schemes, shots_per_scheme=shots, reduced=[2], _tqdm_disable=True)
    from MPDOSimulator.QuantumGates.SingleGates import MeasureX, MeasureY
    kept = [0, 1, 3, 4, 5]
    for s, bits in zip(schemes, out):
        ch = c._chain.clone()
        for q, b in zip(kept, s):
            if b < 2:
                ch.apply_1q(q, c._np((MeasureX if b == 0 else MeasureY)(dtype=c.dtype).tensor))
        p = np.asarray(ch.probs(kept))
        _check_freq(np.array(bits), p / p.sum(), shots)


def test_random_sample_bool_and_argument_errors(S):
    c = _noisy(S)
    out = c.randomSample([[2] * 6], shots_per_scheme=16, _require_bool_result=True, _tqdm_disable=True)
    assert len(out) == 1 and len(out[0]) == 16 and all(isinstance(x, bool) for x in out[0][0])
    assert c.randomSample([], shots_per_scheme=4) == []
    with pytest.raises(ValueError):
        c.randomSample([[2] * 5], shots_per_scheme=4)
    with pytest.raises(Exception, match='basis'):
        c._chain.sample_schemes(list(range(6)), [[3] * 6], 4, [1])
