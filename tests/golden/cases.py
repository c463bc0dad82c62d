"""Golden-fixture circuits, written once against the reference's public
``MPDOSimulator`` API (Circuit.py / AbstractCircuit.py / NoiseChannel.py /
Tools.py).  The same functions run against the reference (make_golden.py,
CPU) and against the GB300 drop-in package (tests/test_golden_gpu.py), so the
two are driven by identical calls.

Every case builds its circuit (gate queue and noise settings);
``evolve_case`` runs it from |0...0> (``Tools.create_ket0Series``) and
``readout`` takes the full density matrix (``cal_dm``, n <= 6) and the
dimensions of every leg of the final state (bond, physics and Kraus legs),
both gauge-invariant.
"""
import math
import os
from typing import Dict

import numpy as np
import torch


def _amplitude_damping(gamma: float, dtype, device) -> torch.Tensor:
    # [out, in, k] layout of NoiseChannel.decay (NoiseChannel.py:144-155)
    k = np.array([[[1, 0], [0, math.sqrt(1 - gamma)]], [[0, math.sqrt(gamma)], [0, 0]]], dtype=np.complex128)
    return torch.as_tensor(np.transpose(k, (1, 2, 0))).to(dtype=dtype, device=device)


def _override_noise(c, p1: float, gamma: float, p2: float, dtype):
    nz = c.Noise
    nz.dephasingTensor = nz.depolarization_noise_channel(p=p1)
    nz.decayTensor = _amplitude_damping(gamma, dtype, nz.dephasingTensor.device)
    nz.dpCTensor2 = nz.depolarization_noise_channel(p=p2, qn=2)


def _connect(c, n: int):
    """Noiseless CZ on every neighbouring pair of |0...0>: the chain gets
    dimension-1 bonds, so truncation is not skipped (Circuit.py:476 checks
    connectivity) and the Kraus legs do not grow unbounded before it."""
    for q in range(n - 1):
        c.cz(q, q + 1, True)
    c.truncate()


def _brickwork(c, n: int, depth: int, seed: int, two_q=('CZ', 'CNOT'), truncate_1q: bool = True):
    """U3 on every qubit (angles U[0, 2pi)), then CZ/CNOT on brickwork pairs
    (alternating even/odd, some with the larger qubit first), truncate after
    every sublayer."""
    rng = np.random.default_rng(seed)
    for L in range(depth):
        for q in range(n):
            th, ph, la = (rng.random(3) * 2 * math.pi).tolist()
            c.u3(th, ph, la, [q])
        if truncate_1q:
            c.truncate()
        for q in range(L % 2, n - 1, 2):
            name = two_q[int(rng.integers(len(two_q)))]
            a, b = (q, q + 1) if rng.random() < 0.7 else (q + 1, q)
            getattr(c, name.lower())(a, b)
        c.truncate()


def noisy_err(S, dtype, device, workdir):
    """idealNoise with the benchmark circuits' noise model (1q depolarising + amplitude
    damping, 2q depolarising) at strong rates; no chi cap, a relative
    truncation error 1e-3 (decompositions.py:121-134 rule, exact SVD) and a
    kappa=2 Kraus cap."""
    c = S.TensorCircuit(4, ideal=False, noiseType='idealNoise', chi=None, kappa=2, max_truncation_err=1e-3,
                        dtype=dtype, device=device)
    _override_noise(c, 0.03, 0.05, 0.08, dtype)
    _connect(c, 4)
    _brickwork(c, 4, 3, seed=11)
    return c


def noisy_chi(S, dtype, device, workdir):
    """idealNoise, chi=4 and kappa=2 caps on n=5 (the reference's randomized
    SVD path runs on its larger bonds)."""
    c = S.TensorCircuit(5, ideal=False, noiseType='idealNoise', chi=4, kappa=2, dtype=dtype, device=device)
    _override_noise(c, 0.02, 0.03, 0.05, dtype)
    _connect(c, 5)
    _brickwork(c, 5, 3, seed=12)
    return c


def ideal_chi(S, dtype, device, workdir):
    """Noiseless circuit (no Kraus legs), chi=2 truncation on n=6."""
    c = S.TensorCircuit(6, ideal=True, chi=2, dtype=dtype, device=device)
    c.h(0)
    _brickwork(c, 6, 3, seed=13)
    return c


def unified_chip(S, dtype, device, workdir):
    """noiseType='unified' with the default chip's decay / dephasing channels
    on 1q gates only (Circuit.py:141), relative error cap 1e-6, kappa=3."""
    c = S.TensorCircuit(4, ideal=False, noiseType='unified', chi=None, kappa=3, max_truncation_err=1e-6,
                        dtype=dtype, device=device)
    rng = np.random.default_rng(14)
    _connect(c, 4)
    c.h(0)
    for q in range(3):
        c.cnot(q, q + 1)
    c.truncate()
    for q in range(4):
        c.rx(float(rng.random() * 2 * math.pi), [q])
        c.ry(float(rng.random() * 2 * math.pi), [q])
    c.truncate()
    for q in (0, 2):
        c.cz(q, q + 1)
    c.s([1])
    c.t([3])
    c.truncate()
    return c


def real_noise(S, dtype, device, workdir):
    """noiseType='realNoise': CZ becomes CZEXP, whose Kraus set is read from a
    chi matrix (RealNoise.py:22-179).  The chi matrix is a seeded synthetic
    Hermitian positive matrix written to an .npz file (key 'chi'), near the
    identity process."""
    rng = np.random.default_rng(15)
    g = 0.15 * (rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16)))
    g[0, 0] += 1.0
    chi = g @ g.conj().T
    chi /= np.trace(chi).real
    fn = os.path.join(workdir, 'chi_cz_synthetic.npz')
    np.savez(fn, chi=chi)
    files = {'CZ': {'01': fn, '12': fn, '23': fn}}
    c = S.TensorCircuit(4, ideal=False, noiseType='realNoise', chiFileDict=files, chi=None, kappa=4,
                        max_truncation_err=1e-8, dtype=dtype, device=device)
    # (no noiseless connecting layer here: in realNoise mode the reference
    # gives an ideal CZ a fifth axis name, Circuit.py:86-87, and fails)
    for q in range(4):
        c.h([q])
    c.truncate()
    c.cz(0, 1)
    c.cz(2, 3)
    c.truncate()
    c.cz(1, 2)
    c.truncate()
    c.cnot(0, 1)
    c.truncate()
    return c


def gate_zoo(S, dtype, device, workdir):
    """idealNoise (the 'medium' chip's 1q channels replaced by the benchmark
    circuits' noise model) over every gate method of the API: fixed and
    parameterised 1q gates, an arbitrary 1q matrix, noisy fixed 2q gates in
    both orientations and parameterised 2q gates (ideal: the reference's
    idealNoise path fails on noisy parameterised 2q gates, AbstractGate axis
    names), then X / Y measurement basis changes and a reset, truncate after
    every sublayer, relative error cap 1e-7."""
    c = S.TensorCircuit(4, ideal=False, noiseType='idealNoise', chi=None, kappa=4, max_truncation_err=1e-7,
                        chip='medium', dtype=dtype, device=device)
    _override_noise(c, 0.02, 0.03, 0.04, dtype)
    _connect(c, 4)
    c.h([0, 3])
    c.x([1])
    c.y([2])
    c.truncate()
    c.z([0])
    c.s([1])
    c.sdg([2])
    c.t([3])
    c.truncate()
    c.rx(0.7, [0])
    c.ry(1.3, [1])
    c.rz(-2.2, [2])
    c.p(0.4, [3])
    c.u1(2.5, [0])
    c.u3(0.9, 1.7, -0.6, [1])
    th = 0.8
    arb = torch.tensor([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]], dtype=dtype)
    c.arbSingle(arb, [2])
    c.truncate()
    c.cy(1, 0)
    c.swap(2, 3)
    c.truncate()
    c.iswap(1, 2)
    c.ii(0, 1, True)
    c.truncate()
    c.cx(3, 2)
    c.rxx(0.5, 0, 1, True)
    c.truncate()
    c.ryy(-1.2, 1, 2, True)
    c.rzz(2.1, 2, 3, True)
    c.truncate()
    c.pswap(0.8, 0, 1, True)
    c.cp(1.9, 3, 2, True)
    c.truncate()
    c.xx_yy(0.6, 0.25, 1, 2, True)
    c.truncate()
    c.measure([0, 2], [0, 1])
    c.reset1([3])
    c.truncate()
    return c


def real_noise_cp(S, dtype, device, workdir):
    """noiseType='realNoise' with CP gates, whose Kraus set comes from a CP
    chi matrix (AbstractCircuit.py:404-421, RealNoise.py cpExp_channel), and
    the 'best' chip's 1q channels."""
    rng = np.random.default_rng(16)
    g = 0.12 * (rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16)))
    g[0, 0] += 1.0
    chi = g @ g.conj().T
    chi /= np.trace(chi).real
    fn = os.path.join(workdir, 'chi_cp_synthetic.npz')
    np.savez(fn, chi=chi)
    files = {'CZ': {}, 'CP': {'01': fn, '12': fn, '23': fn}}
    c = S.TensorCircuit(4, ideal=False, noiseType='realNoise', chiFileDict=files, chi=None, kappa=4,
                        max_truncation_err=1e-8, chip='best', dtype=dtype, device=device)
    for q in range(4):
        c.h([q])
    c.truncate()
    c.cp(None, 0, 1)
    c.cp(None, 3, 2)
    c.truncate()
    c.cp(None, 2, 1)
    c.truncate()
    c.rx(0.4, [0, 1, 2, 3])
    c.truncate()
    return c


CASES = {
    'noisy_err_c128': (noisy_err, torch.complex128),
    'noisy_err_c64': (noisy_err, torch.complex64),
    'noisy_chi_c128': (noisy_chi, torch.complex128),
    'ideal_chi_c128': (ideal_chi, torch.complex128),
    'unified_chip_c128': (unified_chip, torch.complex128),
    'real_noise_c128': (real_noise, torch.complex128),
}

# Cases pinned on the CPU only: the drop-in API builds the reference's
# operations (tests/test_golden_builders.py) and the oracle reproduces the
# reference's density matrix from them (tests/test_golden_oracle.py).  The
# engine runs such operations through the same entry points as CASES; these
# were added after the last GPU run and have not been through the GPU tests.
def unified_medium(S, dtype, device, workdir):
    """noiseType='unified' with the 'medium' chip's decay and dephasing
    channels (ChipInfo.py, NoiseChannel.py:144-170) on every 1q gate."""
    c = S.TensorCircuit(4, ideal=False, noiseType='unified', chi=3, kappa=2, chip='medium', dtype=dtype,
                        device=device)
    _connect(c, 4)
    _brickwork(c, 4, 2, seed=17)
    return c


def unified_best(S, dtype, device, workdir):
    """noiseType='unified' with the 'best' chip: zero bath rate, so its decay
    and dephasing Kraus sets carry exactly-zero operators (rank-deficient
    Kraus legs for the kappa pass)."""
    c = S.TensorCircuit(4, ideal=False, noiseType='unified', chi=4, kappa=2, chip='best', dtype=dtype,
                        device=device)
    _connect(c, 4)
    _brickwork(c, 4, 2, seed=18)
    return c


HOST_CASES = {
    'unified_best_c128': (unified_best, torch.complex128),
    'unified_medium_c128': (unified_medium, torch.complex128),
    'gate_zoo_c128': (gate_zoo, torch.complex128),
    'real_noise_cp_c128': (real_noise_cp, torch.complex128),
}


def evolve_case(S, c, dtype):
    c.evolve(S.Tools.create_ket0Series(c.qnumber, dtype=dtype))
    return c


# dmOperations.pauli_expect terms pinned with every case (observables as
# PAULI_DICT indices 0: X, 1: Y, 2: Z, on the given qubits, one list out of
# order).  dmOperations.expect cannot be pinned: it starts from
# `Tensor(0.)` (dmOperations.py:141), which current torch rejects.
PAULI_TERMS = [([2], [0]), ([0, 1], [1, 2]), ([2, 2], [0, 3]), ([1, 0, 2], [3, 0, 1])]


def readout(c, S=None) -> Dict[str, np.ndarray]:
    dm = c.cal_dm()
    dims = []
    for node in c.stateNodes:
        dims.append({name: int(node.tensor.shape[i]) for i, name in enumerate(node.axis_names)})
    out = {'dm': dm.detach().cpu().numpy(), 'dims': dims}
    if S is not None:
        dmn = c.cal_dmNodes()
        out['pauli'] = np.array([float(S.dmOperations.pauli_expect(dmn, obs, oqs)) for obs, oqs in PAULI_TERMS])
    return out
