"""Noise-channel fitting on the gradient oracle: the checker for the
channel-fitting workload.

TEST INFRASTRUCTURE ONLY; the product never imports it.

Workload (defined here in full, at any size):

* a hidden two-qubit CPTP channel as a rank-4 Kraus set {K_k}, four 4 x 4
  complex matrices whose stack (16 x 4) is an isometry, i.e.
  sum_k K_k^H K_k = I; drawn near the identity channel: the isometry is the
  orthonormalised [I; 0; 0; 0] + eps G with G complex Gaussian from
  ``torch.Generator().manual_seed(seed)``;
* it acts after every CZ.  In reference terms this is realNoise mode with
  ``_cz_expTensors[pair]`` = Kraus o CZ as a (2, 2, 2, 2, 4) tensor
  (AbstractCircuit.py:313-330, Circuit.py:88-89);
* random circuits: per layer a U3 sublayer (angles ~ U[0, 2pi)) and a CZ
  brickwork sublayer (even pairs on even layers, odd pairs on odd layers),
  each followed by ``truncate()``; single-qubit gates ideal;
* data: the single-qubit Z marginals <Z_i> of every circuit under the hidden
  channel;
* model: a trainable Kraus set on the Stiefel manifold (the orthonormal
  factor of an unconstrained 16 x 4 matrix W, QR with a positive R
  diagonal), initialised next to the identity channel, fitted by Adam on the
  squared error of the marginals through the gradient oracle
  (``oracle.adjoint``: reverse mode through the truncating evolution);
* error measure: the diamond-norm proxy || J_fit - J_true ||_1 / 2 (trace
  norm of the difference of the trace-one Choi matrices).
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional

import numpy as np
import torch

from . import mpdo_oracle as O
from . import adjoint as A

_CZ = O.gate_2q('CZ').reshape(4, 4)


def hidden_isometry(seed: int = 7, eps: float = 0.05) -> torch.Tensor:
    """16 x 4 isometry near [I; 0; 0; 0] (the identity channel)."""
    g = torch.Generator().manual_seed(seed)
    G = torch.complex(torch.randn(16, 4, dtype=torch.float64, generator=g),
                      torch.randn(16, 4, dtype=torch.float64, generator=g)) / math.sqrt(2)
    X = torch.zeros(16, 4, dtype=torch.complex128)
    X[:4] = torch.eye(4, dtype=torch.complex128)
    return stiefel(X + eps * G)


def stiefel(W: torch.Tensor) -> torch.Tensor:
    """Orthonormal factor of W with a positive R diagonal (unique for full
    column rank; differentiable)."""
    Q, R = torch.linalg.qr(W)
    d = torch.diagonal(R)
    ph = torch.where(d.abs() > 0, d / d.abs(), torch.ones_like(d))
    return Q * ph[None, :]


def kraus(V: torch.Tensor) -> torch.Tensor:
    """Kraus operators [k, out, in] of a 16 x 4 isometry (rows k-major)."""
    return V.reshape(4, 4, 4)


def cz_channel_tensor(K: torch.Tensor) -> torch.Tensor:
    """Kraus o CZ as [o0, o1, i0, i1, k] (the realNoise 2q layout)."""
    t = torch.einsum('kom,mi->oik', K, _CZ.to(K.dtype))       # [out, in, k]
    return t.reshape(2, 2, 2, 2, 4)


def choi(K: torch.Tensor) -> torch.Tensor:
    """Trace-one Choi matrix sum_k vec(K_k) vec(K_k)^H / 4 (16 x 16)."""
    v = K.reshape(4, 16)                                      # vec row-major per Kraus operator
    return torch.einsum('ka,kb->ab', v, v.conj()) / 4


def diamond_proxy(K_fit: torch.Tensor, K_true: torch.Tensor) -> float:
    """|| J_fit - J_true ||_1 / 2 (Hermitian difference: half the sum of |eigenvalues|)."""
    d = choi(K_fit.detach()) - choi(K_true.detach())
    return float(torch.linalg.eigvalsh(d).abs().sum() / 2)


def random_circuit(n: int, depth: int, seed: int) -> torch.Tensor:
    """U3 angles [depth, n, 3] ~ U[0, 2pi) from ``torch.Generator().manual_seed(seed)``."""
    g = torch.Generator().manual_seed(seed)
    return 2 * math.pi * torch.rand(depth, n, 3, dtype=torch.float64, generator=g)


def circuit_ops(angles: torch.Tensor, cz_t: torch.Tensor) -> list:
    depth, n, _ = angles.shape
    ops = []
    for l in range(depth):
        ops += [('1q', q, A.u3(angles[l, q, 0], angles[l, q, 1], angles[l, q, 2])) for q in range(n)]
        ops.append(('truncate',))
        ops += [('2q', q, q + 1, cz_t) for q in range(l % 2, n - 1, 2)]
        ops.append(('truncate',))
    return ops


_Z = torch.as_tensor(O._PAULI[3].astype(np.complex128))


def marginals(angles: torch.Tensor, K: torch.Tensor, chi: int, kappa: int) -> torch.Tensor:
    """<Z_i> of one circuit under the channel K (unnormalised Tr(rho Z_i))."""
    n = angles.shape[1]
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, circuit_ops(angles, cz_channel_tensor(K)), chi=chi, kappa=kappa, noisy=True)
    return torch.stack([O.expect_ops(st, {i: _Z}) for i in range(n)])


def fit(circuits: List[torch.Tensor], data: List[torch.Tensor], chi: int, kappa: int, steps: int,
        lr: float = 0.02, K_true: Optional[torch.Tensor] = None, init_seed: int = 1,
        init_eps: float = 1e-2) -> Dict[str, list]:
    """Adam on W (16 x 4 complex) minimising sum_c || <Z>_c(stiefel(W)) -
    data_c ||^2.  W starts at ``hidden_isometry(init_seed, init_eps)``, the
    identity channel moved by ``init_eps``.  The exact identity
    (``init_eps = 0``) runs -- the gradient oracle keeps the numerical rank
    of its rank-deficient bonds -- but it is a stationary point of every
    dissipative direction: rho depends on the three zero Kraus operators
    quadratically, so their gradient vanishes there and Adam could only fit
    a unitary.  Returns the loss per step (before the update) and, with
    ``K_true``, the diamond-norm proxy."""
    W = hidden_isometry(seed=init_seed, eps=init_eps).clone().requires_grad_(True)
    opt = torch.optim.Adam([W], lr=lr)
    hist = {'loss': [], 'proxy': []}
    for _ in range(steps):
        opt.zero_grad()
        K = kraus(stiefel(W))
        loss = sum(((marginals(a, K, chi, kappa) - d) ** 2).sum() for a, d in zip(circuits, data))
        loss.backward()
        hist['loss'].append(float(loss.detach()))
        if K_true is not None:
            hist['proxy'].append(diamond_proxy(K, K_true))
        opt.step()
    K = kraus(stiefel(W.detach()))
    hist['loss'].append(float(sum(((marginals(a, K, chi, kappa) - d) ** 2).sum()
                                  for a, d in zip(circuits, data))))
    if K_true is not None:
        hist['proxy'].append(diamond_proxy(K, K_true))
    hist['W'] = W.detach()
    return hist
