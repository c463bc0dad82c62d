"""Seeded synthetic circuits of the benchmark configurations.

A circuit is a list of layers:
  ('1q', name, params, qubit)      single-qubit gate followed by its noise
  ('2q', name, params, q0, q1)     nearest-neighbour gate followed by 2q noise
  ('truncate',)
plus a noise spec {p1: 1q depolarising, gamma: amplitude damping, p2: 2q
depolarising}.  After every 1q gate the channel is depolarising(p1) then
amplitude damping(gamma) (the reference's dephasing and decay slots,
Circuit.py:146-155); after every 2q gate depolarising(p2)
(Circuit.py:91-100).  A truncate() follows every gate sublayer.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List

import numpy as np
import torch


@dataclass
class Workload:
    name: str
    n: int
    chi: int
    kappa: int
    layers: List[tuple]
    noise: dict = field(default_factory=lambda: dict(p1=1e-3, gamma=1e-3, p2=1e-2))
    depth: int = 0

    @property
    def gates(self) -> int:
        return sum(1 for L in self.layers if L[0] in ('1q', '2q'))

    @property
    def gate_layers(self) -> int:
        return sum(1 for L in self.layers if L[0] == 'truncate')


def ry_rz_cnot_brickwork(n: int = 8, depth: int = 8, chi: int = 16, kappa: int = 4) -> Workload:
    """n=8, 8 brickwork layers of RY(theta), RZ(phi) on every qubit then CNOT on
    even/odd pairs alternating; angles U[0, 2pi) from torch.Generator seed 0
    drawn layer -> sublayer -> qubit in float64."""
    g = torch.Generator().manual_seed(0)
    layers = []
    for L in range(depth):
        for name in ('RY', 'RZ'):
            ang = (torch.rand(n, generator=g, dtype=torch.float64) * 2 * math.pi).tolist()
            layers += [('1q', name, (ang[q],), q) for q in range(n)]
            layers.append(('truncate',))
        layers += [('2q', 'CNOT', (), q, q + 1) for q in range(L % 2, n - 1, 2)]
        layers.append(('truncate',))
    return Workload(f'n={n} depth={depth} RY/RZ/CNOT brickwork, chi={chi} kappa={kappa}', n, chi, kappa, layers, depth=depth)


def u3_brickwork(n: int = 32, depth: int = 20, chi: int = 64, kappa: int = 4, seed: int = 0) -> Workload:
    """n=32, depth 20: U3 (angles U[0, 2pi)) on every qubit, then CZ or CNOT
    (p = 0.5 each) on brickwork pairs alternating even/odd; seed 0."""
    g = torch.Generator().manual_seed(seed)
    layers = []
    for L in range(depth):
        ang = (torch.rand(n, 3, generator=g, dtype=torch.float64) * 2 * math.pi).tolist()
        layers += [('1q', 'U3', tuple(ang[q]), q) for q in range(n)]
        layers.append(('truncate',))
        pairs = list(range(L % 2, n - 1, 2))
        pick = torch.rand(len(pairs), generator=g, dtype=torch.float64).tolist()
        layers += [('2q', 'CZ' if u < 0.5 else 'CNOT', (), q, q + 1) for u, q in zip(pick, pairs)]
        layers.append(('truncate',))
    return Workload(f'n={n} depth={depth} U3 + CZ/CNOT brickwork, chi={chi} kappa={kappa}', n, chi, kappa,
                    layers, depth=depth)


def uneven_batch_circuit(seed: int) -> Workload:
    """One circuit of the uneven batch: n ~ U{12..40}, depth ~ U{10..30},
    chi from {16, 32, 64, 128}, kappa from {2, 4}, drawn from
    torch.Generator seed ``seed``; gates and noise as the n=32 workload (its
    angles and gate picks continue from the same generator's seed)."""
    g = torch.Generator().manual_seed(int(seed))
    n = int(torch.randint(12, 41, (1,), generator=g))
    depth = int(torch.randint(10, 31, (1,), generator=g))
    chi = (16, 32, 64, 128)[int(torch.randint(0, 4, (1,), generator=g))]
    kappa = (2, 4)[int(torch.randint(0, 2, (1,), generator=g))]
    w = u3_brickwork(n=n, depth=depth, chi=chi, kappa=kappa, seed=int(seed))
    w.name = f'uneven batch circuit seed={seed}: n={n} depth={depth} chi={chi} kappa={kappa}'
    return w


def amplitude_damping(gamma: float) -> np.ndarray:
    k = np.array([[[1, 0], [0, math.sqrt(1 - gamma)]], [[0, math.sqrt(gamma)], [0, 0]]], dtype=np.complex128)
    return np.transpose(k, (1, 2, 0))


def build_circuit(w: Workload, dtype=torch.complex64, device=None):
    """The workload as a drop-in ``TensorCircuit`` (noiseType='idealNoise' with
    the noise tensors overridden, as the reference allows)."""
    from MPDOSimulator import TensorCircuit
    c = TensorCircuit(w.n, ideal=False, noiseType='idealNoise', chi=w.chi, kappa=w.kappa, dtype=dtype,
                      device=device)
    nz = c.Noise
    nz.dephasingTensor = nz.depolarization_noise_channel(p=w.noise['p1'])
    nz.decayTensor = torch.as_tensor(amplitude_damping(w.noise['gamma'])).to(dtype=dtype, device=nz.device)
    nz.dpCTensor2 = nz.depolarization_noise_channel(p=w.noise['p2'], qn=2)
    for L in w.layers:
        if L[0] == 'truncate':
            c.truncate()
        elif L[0] == '1q':
            _, name, p, q = L
            getattr(c, name.lower())(*p, q)
        else:
            _, name, p, q0, q1 = L
            getattr(c, name.lower())(*p, q0, q1)
    return c
