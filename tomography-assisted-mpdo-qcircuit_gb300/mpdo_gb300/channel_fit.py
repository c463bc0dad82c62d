"""Fitting a two-qubit noise channel to Z-basis marginals with the GPU
adjoint: many independent circuits, forward and reverse sweeps on the GPU,
the Kraus set trained on the Stiefel manifold by Adam.

Workload: a hidden two-qubit CPTP channel (rank-4 Kraus set: four 4 x 4
matrices whose 16 x 4 stack is an isometry) acts after every CZ of random
circuits -- per layer a U3 sublayer (ideal gates, angles U[0, 2pi)) and a CZ
brickwork sublayer, a truncate() after each.  In reference terms this is
realNoise mode with ``_cz_expTensors[pair]`` = Kraus o CZ as a
(2, 2, 2, 2, 4) tensor (AbstractCircuit.py:313-330, Circuit.py:88-89).  The
data are the circuits' marginals <Z_i>; the model is the orthonormal factor
(positive R diagonal) of an unconstrained 16 x 4 matrix W; the error measure
the diamond-norm proxy ||J_fit - J_true||_1 / 2 of the trace-one Choi
matrices.

``Marginals`` is a torch.autograd.Function: its forward evolves every circuit
and returns their <Z_i> (batched engine), its backward runs the engine's
adjoint once per circuit with H = sum_i gbar_i Z_i -- the incoming cotangent
of the marginals -- so any loss of the marginals trains the Kraus set.  The
circuits' adjoints run concurrently on separate engines (each on its own
stream; the C calls release the GIL).
"""
from __future__ import annotations

import concurrent.futures as cf
import math
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import adjoint as AD
from .engine import Batch, Engine

CZ = torch.diag(torch.tensor([1, 1, 1, -1], dtype=torch.complex128))


def hidden_isometry(seed: int = 7, eps: float = 0.05) -> torch.Tensor:
    """16 x 4 isometry: the orthonormalised [I; 0; 0; 0] + eps G, G complex
    Gaussian (re, im ~ N(0, 1/2)) from ``torch.Generator().manual_seed(seed)``."""
    g = torch.Generator().manual_seed(seed)
    G = torch.complex(torch.randn(16, 4, dtype=torch.float64, generator=g),
                      torch.randn(16, 4, dtype=torch.float64, generator=g)) / math.sqrt(2)
    X = torch.zeros(16, 4, dtype=torch.complex128)
    X[:4] = torch.eye(4, dtype=torch.complex128)
    return stiefel(X + eps * G)


def stiefel(W: torch.Tensor) -> torch.Tensor:
    """Orthonormal factor of W with a positive R diagonal (differentiable)."""
    Q, R = torch.linalg.qr(W)
    d = torch.diagonal(R)
    ph = torch.where(d.abs() > 0, d / d.abs(), torch.ones_like(d))
    return Q * ph[None, :]


def kraus(V: torch.Tensor) -> torch.Tensor:
    """Kraus operators [k, out, in] of a 16 x 4 isometry (rows k-major)."""
    return V.reshape(4, 4, 4)


def cz_channel_tensor(K: torch.Tensor) -> torch.Tensor:
    """Kraus o CZ as [o0, o1, i0, i1, k] (the realNoise 2q layout)."""
    t = torch.einsum('kom,mi->oik', K, CZ.to(K.dtype))
    return t.reshape(2, 2, 2, 2, 4)


def choi(K: torch.Tensor) -> torch.Tensor:
    """Trace-one Choi matrix sum_k vec(K_k) vec(K_k)^H / 4."""
    v = K.reshape(4, 16)
    return torch.einsum('ka,kb->ab', v, v.conj()) / 4


def diamond_proxy(K_fit: torch.Tensor, K_true: torch.Tensor) -> float:
    """||J_fit - J_true||_1 / 2 (half the sum of the difference's |eigenvalues|)."""
    d = choi(K_fit.detach()) - choi(K_true.detach())
    return float(torch.linalg.eigvalsh(d).abs().sum() / 2)


def random_angles(n: int, depth: int, seed: int) -> torch.Tensor:
    """U3 angles [depth, n, 3] ~ U[0, 2pi) from ``torch.Generator().manual_seed(seed)``."""
    g = torch.Generator().manual_seed(seed)
    return 2 * math.pi * torch.rand(depth, n, 3, dtype=torch.float64, generator=g)


def u3(t, p, l) -> np.ndarray:
    """SingleGates.py:179-185."""
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -np.exp(1j * l) * s], [np.exp(1j * p) * s, np.exp(1j * (l + p)) * c]], dtype=np.complex128)


def circuit_ops(angles: torch.Tensor, cz_t) -> list:
    """Engine ops of one circuit with the 2q tensor ``cz_t`` after every CZ."""
    depth, n, _ = angles.shape
    a = angles.tolist()
    ops = []
    for l in range(depth):
        ops += [('1q', q, u3(*a[l][q])) for q in range(n)]
        ops.append(('truncate',))
        ops += [('2q', q, cz_t) for q in range(l % 2, n - 1, 2)]
        ops.append(('truncate',))
    return ops


class Fitter:
    """Evolves a fixed set of circuits under a trainable 2q channel on one GPU:
    ``marginals(t)`` (differentiable in the (2, 2, 2, 2, 4) channel tensor t)
    returns the [circuits, n] marginals."""

    def __init__(self, circuits: Sequence[torch.Tensor], chi: int, kappa: int, dtype: str = 'complex64',
                 device: int = 0, workers: int = 16):
        self.circuits = list(circuits)
        self.n = int(self.circuits[0].shape[1])
        self.chi, self.kappa, self.dtype = chi, kappa, dtype
        self.batch = Batch.get(device, workers)
        self.engines = [Engine(device) for _ in range(min(workers, len(self.circuits)))]
        self.pool = cf.ThreadPoolExecutor(max_workers=len(self.engines))

    def forward(self, t: np.ndarray) -> np.ndarray:
        progs = [dict(n=self.n, dtype=self.dtype, vectors=[[1, 0]] * self.n, connected=True, chi=self.chi,
                      kappa=self.kappa, max_err=None, noisy=True, ops=circuit_ops(a, t), z=True)
                 for a in self.circuits]
        res = self.batch.run(progs)
        return np.stack([r['z'] for r in res])

    def backward(self, t: np.ndarray, gbar: np.ndarray) -> np.ndarray:
        """sum over circuits and CZ gates of dL/dt for L = sum gbar[c, i] <Z_i>_c."""
        def one(j):
            c = self.circuits[j]
            terms = [(float(gbar[j, i]), {i: 'Z'}) for i in range(self.n) if gbar[j, i] != 0]
            if not terms:
                return np.zeros((2, 2, 2, 2, 4), dtype=np.complex128)
            ops = circuit_ops(c, t)
            eng = self.engines[j % len(self.engines)]
            _, grads = AD.program_grad(ops, self.n, terms, self.chi, self.kappa, dtype=self.dtype, engine=eng)
            return sum(g for op, g in zip(ops, grads) if op[0] == '2q')
        # circuits sharing an engine run one after another on its worker
        groups = [list(range(w, len(self.circuits), len(self.engines))) for w in range(len(self.engines))]
        out = np.zeros((2, 2, 2, 2, 4), dtype=np.complex128)
        for part in self.pool.map(lambda js: sum(one(j) for j in js), groups):
            out += part
        return out

    def marginals(self, t: torch.Tensor) -> torch.Tensor:
        return _Marginals.apply(self, t)


class _Marginals(torch.autograd.Function):
    @staticmethod
    def forward(ctx, fitter, t):
        tn = t.detach().cpu().to(torch.complex128).numpy()
        ctx.fitter, ctx.tn = fitter, tn
        ctx.dtype, ctx.device = t.dtype, t.device
        return torch.from_numpy(fitter.forward(tn))

    @staticmethod
    def backward(ctx, gout):
        g = ctx.fitter.backward(ctx.tn, gout.detach().cpu().numpy().astype(np.float64))
        return None, torch.from_numpy(g).to(dtype=ctx.dtype, device=ctx.device)


def _allreduce_sum(x: torch.Tensor, group) -> torch.Tensor:
    import torch.distributed as dist
    r = torch.view_as_real(x) if x.is_complex() else x
    dist.all_reduce(r, op=dist.ReduceOp.SUM, group=group)
    return x


def fit(fitter: Fitter, data: torch.Tensor, steps: int, lr: float = 0.02, K_true: Optional[torch.Tensor] = None,
        init_seed: int = 1, init_eps: float = 1e-2, callback=None, group=None):
    """Adam on W (16 x 4 complex) minimising sum_c ||<Z>_c - data_c||^2,
    starting from the identity channel moved by ``init_eps`` (the exact
    identity is stationary for every dissipative direction).  Returns the
    loss per step (before the update) and, with ``K_true``, the proxy.

    Over several GPUs each rank passes a ``fitter`` over its own circuits
    (and their ``data`` rows) and a process ``group``: the loss and the
    gradient of W (64 complex numbers) are summed over the group once per
    step, so every rank takes the same Adam step from the same W."""
    W = hidden_isometry(seed=init_seed, eps=init_eps).clone().requires_grad_(True)
    opt = torch.optim.Adam([W], lr=lr)
    hist = {'loss': [], 'proxy': []}
    for step in range(steps):
        opt.zero_grad()
        K = kraus(stiefel(W))
        m = fitter.marginals(cz_channel_tensor(K))
        loss = ((m - data) ** 2).sum()
        loss.backward()
        if group is not None:
            _allreduce_sum(W.grad, group)
            loss = _allreduce_sum(loss.detach().clone(), group)
        hist['loss'].append(float(loss.detach()))
        if K_true is not None:
            hist['proxy'].append(diamond_proxy(K, K_true))
        opt.step()
        if callback:
            callback(step, hist)
    hist['W'] = W.detach()
    return hist
