"""Gradients of expectation values through the GPU engine's hand-written
adjoint (``mpdo_program_grad`` in include/mpdo_gb300.h).

``program_loss(ops, n, terms, ...)`` evolves a circuit given as engine
operations -- ('1q', site, kraus[2,2,K]), ('2q', site_min,
kraus[o_min,o_max,i_min,i_max,K]), ('truncate',), ('kappa',) -- whose Kraus
tensors are torch tensors, and returns L = sum_t c_t Re Tr(rho P_t) as a
torch scalar.  Its backward is the engine's reverse sweep (checkpointed per
truncate layer), so gradients flow into whatever built the Kraus tensors:
gate angles, noise probabilities, Stiefel-parameterised Kraus sets.

The reference has no gradient of its own: its gate tensors are rebuilt by
``torch.tensor(data=...)`` and detach the angles (SingleGates.py:181-185,
YGates.py:66-68).  What is differentiated here is its evolution
(Circuit.py:469-491, TNNOptimizer.py:87-197) in the engine's order, with
every split keeping at most its numerical rank (``rank_tol``).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import check
from .engine import Engine, _cplx, _dptr

_PAULI = {
    'I': np.eye(2, dtype=np.complex128),
    'X': np.array([[0, 1], [1, 0]], dtype=np.complex128),
    'Y': np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    'Z': np.array([[1, 0], [0, -1]], dtype=np.complex128),
}
_CODE = {0: 'I', 1: 'X', 2: 'Y', 3: 'Z'}

DEFAULT_RANK_TOL = {'complex64': 1e-5, 'complex128': 1e-13}
DEFAULT_BROADENING = {'complex64': 1e-6, 'complex128': 1e-12}


def pauli_mpo(n: int, terms: Sequence[Tuple[float, Dict[int, object]]]) -> Tuple[np.ndarray, np.ndarray]:
    """Matrix-product operator of H = sum_t c_t prod_{q in t} P_{t,q} (real
    c_t, Paulis 'I'/'X'/'Y'/'Z' or codes 0..3): the finite-state form with a
    'not started' and a 'done' channel on every bond plus one channel per
    term whose support spans the bond.  Returns (dims[n + 1], W) with W the
    concatenation over sites of W_k[D_k][D_k+1][out][in]."""
    parsed = []
    for c, ops in terms:
        ops = {int(q): (_CODE[p] if isinstance(p, (int, np.integer)) else str(p).upper()) for q, p in ops.items()}
        ops = {q: p for q, p in ops.items() if p != 'I'}
        if not ops:
            raise ValueError('a term needs at least one non-identity Pauli (constants do not depend on the state)')
        if min(ops) < 0 or max(ops) >= n:
            raise ValueError('Pauli term acts outside the chain')
        parsed.append((float(c), ops, min(ops), max(ops)))

    def chans(k):               # channels of bond k (between sites k-1 and k)
        if k == 0:
            return ['start']
        if k == n:
            return ['done']
        return ['start', 'done'] + [t for t, (_, _, lo, hi) in enumerate(parsed) if lo < k <= hi]
    dims = np.array([len(chans(k)) for k in range(n + 1)], dtype=np.int32)
    blocks = []
    eye = _PAULI['I']
    for k in range(n):
        left, right = chans(k), chans(k + 1)
        W = np.zeros((len(left), len(right), 2, 2), dtype=np.complex128)
        li, ri = {c: i for i, c in enumerate(left)}, {c: i for i, c in enumerate(right)}
        if 'start' in li and 'start' in ri:
            W[li['start'], ri['start']] = eye
        if 'done' in li and 'done' in ri:
            W[li['done'], ri['done']] = eye
        for t, (c, ops, lo, hi) in enumerate(parsed):
            if not lo <= k <= hi:
                continue
            P = _PAULI[ops.get(k, 'I')]
            src = li['start'] if k == lo else li[t]
            dst = ri['done'] if k == hi else ri[t]
            W[src, dst] += (c if k == lo else 1.0) * P
        blocks.append(W.ravel())
    return dims, np.concatenate(blocks)


def _flatten(ops) -> tuple:
    kinds = {'1q': _lib.MPDO_OP_1Q, '2q': _lib.MPDO_OP_2Q, 'truncate': _lib.MPDO_OP_TRUNCATE,
             'kappa': _lib.MPDO_OP_KAPPA}
    kind = np.array([kinds[o[0]] for o in ops], dtype=np.int32)
    site = np.array([o[1] if len(o) > 1 else 0 for o in ops], dtype=np.int32)
    tens = []
    for o in ops:
        if len(o) > 2:
            t = o[2].detach().to('cpu', torch.complex128).numpy() if torch.is_tensor(o[2]) else \
                np.asarray(o[2], dtype=np.complex128)
            t = t[..., None] if t.ndim in (2, 4) else t
            tens.append(np.ascontiguousarray(t))
        else:
            tens.append(None)
    kk = np.array([t.shape[-1] if t is not None else 1 for t in tens], dtype=np.int32)
    sizes = [2 * t.size if t is not None else 0 for t in tens]
    off = np.zeros(len(ops), dtype=np.int64)
    if len(ops) > 1:
        off[1:] = np.cumsum(sizes[:-1])
    flat = np.concatenate([t.view(np.float64).ravel() for t in tens if t is not None]) \
        if any(t is not None for t in tens) else np.zeros(1)
    return kind, site, kk, off, flat, tens


def program_grad(ops, n: int, terms, chi: Optional[int], kappa: Optional[int], dtype: str = 'complex64',
                 noisy: bool = True, vectors=None, rank_tol: Optional[float] = None,
                 broadening: Optional[float] = None, engine: Optional[Engine] = None, timing: Optional[dict] = None):
    """Loss and its gradient with respect to every op's Kraus tensor (a list
    aligned with ``ops``: complex128 arrays shaped like the op's tensor, None
    for truncate / kappa ops), in torch's convention dL/dRe + i dL/dIm.
    ``timing`` (a dict) receives the CUDA-event spans of the forward pass,
    the readout with its adjoint and the reverse sweep, in ms."""
    dtype = 'complex128' if str(dtype).endswith('128') else 'complex64'
    eng = engine or Engine.get(0)
    lib = eng._lib
    kind, site, kk, off, flat, tens = _flatten(ops)
    vec = _cplx(np.asarray(vectors if vectors is not None else [[1, 0]] * n, dtype=np.complex128).reshape(n, 2))
    pr = _lib.Program()
    pr.n, pr.connected = n, 1
    pr.dtype = _lib.MPDO_C128 if dtype == 'complex128' else _lib.MPDO_C64
    pr.vectors = _dptr(vec)
    pr.chi, pr.kappa, pr.max_err, pr.noisy = int(chi or 0), int(kappa or 0), -1.0, int(bool(noisy))
    pr.abs_cutoff = 0.0
    pr.nops = len(ops)
    pr.op_kind = kind.ctypes.data_as(C.POINTER(C.c_int))
    pr.op_site = site.ctypes.data_as(C.POINTER(C.c_int))
    pr.op_k = kk.ctypes.data_as(C.POINTER(C.c_int))
    pr.op_offset = off.ctypes.data_as(C.POINTER(C.c_int64))
    pr.kraus = _dptr(flat)
    pr.z = pr.zz = pr.discarded = None
    dims, W = pauli_mpo(n, terms)
    wbuf = _cplx(W)
    grad = np.zeros_like(flat)
    loss = C.c_double()
    ph = np.zeros(3)
    check(lib.mpdo_program_grad(eng.handle, C.byref(pr), dims.ctypes.data_as(C.POINTER(C.c_int)), _dptr(wbuf),
                                float(rank_tol if rank_tol is not None else DEFAULT_RANK_TOL[dtype]),
                                float(broadening if broadening is not None else DEFAULT_BROADENING[dtype]),
                                C.byref(loss), _dptr(grad), _dptr(ph)))
    if timing is not None:
        timing.update(forward_ms=float(ph[0]), readout_ms=float(ph[1]), reverse_ms=float(ph[2]))
    grads = []
    for j, t in enumerate(tens):
        if t is None:
            grads.append(None)
            continue
        g = grad[off[j]: off[j] + 2 * t.size].view(np.complex128).reshape(t.shape)
        grads.append(g)
    return float(loss.value), grads


class _ProgramLoss(torch.autograd.Function):
    """Forward runs the evolution, the readout and the engine's reverse sweep
    in one call (``mpdo_program_grad``); backward hands the stored Kraus-tensor
    gradients to autograd."""

    @staticmethod
    def forward(ctx, meta, *kraus):
        ops = []
        it = iter(kraus)
        for o in meta['ops']:
            ops.append((o[0], o[1], next(it)) if o[0] in ('1q', '2q') else o)
        loss, grads = program_grad(ops, **meta['kw'])
        ctx.shapes = [k.shape for k in kraus]
        ctx.dtypes = [k.dtype for k in kraus]
        ctx.devices = [k.device for k in kraus]
        ctx.grads = [g for g in grads if g is not None]
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        out = [None]
        for g, shape, dt, dev in zip(ctx.grads, ctx.shapes, ctx.dtypes, ctx.devices):
            gt = torch.from_numpy(np.ascontiguousarray(g)).reshape(shape)
            out.append((gout.detach().cpu().to(torch.float64) * gt).to(dtype=dt, device=dev)
                       if dt.is_complex else None)
        return tuple(out)


def program_loss(ops, n: int, terms, chi: Optional[int], kappa: Optional[int], dtype: str = 'complex64',
                 noisy: bool = True, vectors=None, rank_tol: Optional[float] = None,
                 broadening: Optional[float] = None, engine: Optional[Engine] = None,
                 timing: Optional[dict] = None) -> torch.Tensor:
    """L = sum_t c_t Re Tr(rho P_t) after evolving ``ops`` from the product
    state ``vectors`` (default |0...0>, connected chain), differentiable with
    respect to the ops' Kraus tensors (torch tensors on any device; they are
    read to the host, where they travel as kernel parameters)."""
    kraus = [o[2] if torch.is_tensor(o[2]) else torch.as_tensor(np.asarray(o[2], dtype=np.complex128))
             for o in ops if o[0] in ('1q', '2q')]
    meta = {'ops': [(o[0], o[1]) if o[0] in ('1q', '2q') else o for o in ops],
            'kw': dict(n=n, terms=terms, chi=chi, kappa=kappa, dtype=dtype, noisy=noisy, vectors=vectors,
                       rank_tol=rank_tol, broadening=broadening, engine=engine, timing=timing)}
    return _ProgramLoss.apply(meta, *kraus)


# ---------------------------------------------------------------------------
# differentiable gates and channels for the gradient workloads (the same
# matrices as the drop-in's QuantumGates and NoiseChannel)
# ---------------------------------------------------------------------------
def _c(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.float64).to(torch.complex128)


def ry(theta: torch.Tensor) -> torch.Tensor:
    """YGates.py:65-67."""
    c, s = _c(torch.cos(theta / 2)), _c(torch.sin(theta / 2))
    return torch.stack([torch.stack([c, -s]), torch.stack([s, c])])


def rz(theta: torch.Tensor) -> torch.Tensor:
    """ZGates.py:65-66."""
    e = torch.exp(-0.5j * _c(theta))
    z = torch.zeros((), dtype=torch.complex128)
    return torch.stack([torch.stack([e, z]), torch.stack([z, e.conj()])])


CZ = torch.diag(torch.tensor([1, 1, 1, -1], dtype=torch.complex128)).reshape(2, 2, 2, 2)
_PAULI_T = torch.as_tensor(np.stack([_PAULI[k] for k in 'IXYZ']))


def depolarization(p: torch.Tensor, qn: int = 1) -> torch.Tensor:
    """NoiseChannel.py:51-91 with a differentiable probability: weights
    sqrt(1 - (4^n - 1) p / 4^n) on the identity and sqrt(p / 4^n) on the other
    Pauli strings (kron order, first qubit slowest), layout [out..., in..., k]."""
    d = 4 ** qn
    p = torch.as_tensor(p).to(torch.float64)
    w = torch.cat([torch.sqrt(1 - (d - 1) * p / d).reshape(1), torch.sqrt(p / d).expand(d - 1)])
    ops = _PAULI_T
    for _ in range(qn - 1):
        ops = torch.stack([torch.kron(a, b) for a in ops for b in _PAULI_T])
    t = ops * _c(w)[:, None, None]
    return t.permute(1, 2, 0).reshape([2] * (2 * qn) + [d])


def noisy_1q(g: torch.Tensor, p: Optional[torch.Tensor]) -> torch.Tensor:
    """Depolarising after a 1q gate (the reference's noisy composite,
    Circuit.py:141-155, with the decay slot the identity): [out, in, k]."""
    return g if p is None else torch.einsum('xyk,ys->xsk', depolarization(p, 1), g)


def noisy_2q(g: torch.Tensor, p: Optional[torch.Tensor]) -> torch.Tensor:
    """Circuit.py:95: einsum('ijklp, klmn -> ijmnp'), 2q depolarising after the gate."""
    return g if p is None else torch.einsum('ijklp,klmn->ijmnp', depolarization(p, 2), g)


def hea_ops(angles: torch.Tensor, p: Optional[Dict[str, torch.Tensor]] = None) -> list:
    """Engine ops of the hardware-efficient ansatz: per layer an RY sublayer,
    an RZ sublayer and a CZ ladder (0,1), (1,2), ..., each followed by a
    truncate; one depolarising probability per gate type ('ry', 'rz', 'cz')."""
    layers, _, n = angles.shape
    p = p or {}
    ops = []
    for l in range(layers):
        for j, (gate, key) in enumerate(((ry, 'ry'), (rz, 'rz'))):
            ops += [('1q', q, noisy_1q(gate(angles[l, j, q]), p.get(key))) for q in range(n)]
            ops.append(('truncate',))
        cz = noisy_2q(CZ, p.get('cz'))
        ops += [('2q', q, cz) for q in range(n - 1)]
        ops.append(('truncate',))
    return ops


def ising_terms(n: int, hx: float = 0.5) -> list:
    """sum_i Z_i Z_{i+1} + hx sum_i X_i."""
    return [(1.0, {i: 'Z', i + 1: 'Z'}) for i in range(n - 1)] + [(hx, {i: 'X'}) for i in range(n)]
