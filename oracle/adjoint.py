"""Reverse-mode gradient of the MPDO evolution: the gradient oracle.

TEST INFRASTRUCTURE ONLY (the checker for gradients of expectation values
with respect to gate angles and noise-channel parameters); the product never
imports it.

The reference has no gradient of its own: gate tensors are rebuilt through
``torch.tensor(data=[[...]])`` (SingleGates.py:181-185, YGates.py:66-68,
ZGates.py:66), which detaches them from the angles, and the noise tensors
come from numpy (NoiseChannel.py:76-79, 148-154).  Its evolution is
nevertheless a differentiable function of the gate and Kraus tensors, and
this module differentiates exactly that function -- ``mpdo_oracle.evolve``
with the reference's truncation placement, split cutoff, QR left-to-right
sweep, chi-truncating SVD right-to-left sweep and kappa pass -- by torch
autograd, with

* gate matrices and depolarising Kraus sets built from real parameter
  tensors by differentiable torch ops (same matrices as ``gate_1q`` /
  ``gate_2q`` / ``depolarization``);
* a truncated SVD of its own (``truncated_svd``): forward = the full thin SVD
  and the reference's keep rule; backward = the complex SVD adjoint over ALL
  singular triplets (kept and discarded), the discarded ones entering with a
  zero cotangent, so the gradient is that of the truncated factors, with the
  ``1/(s_j^2 - s_i^2)`` terms broadened to
  ``(s_j^2 - s_i^2) / ((s_j^2 - s_i^2)^2 + eta)`` so that exactly or nearly
  degenerate pairs (whose numerators vanish for a gauge-invariant loss) stay
  finite;
* torch's own QR backward for the left-to-right sweep.  It solves with R^H,
  so it needs full-rank bonds: a bond that keeps exact zero singular values
  (the chi cap keeps them whenever it exceeds the rank,
  decompositions.py:121-140) gives a singular R and NaN gradients.  The
  differentiated splits therefore keep at most the numerical rank
  (singular values above RANK_TOL * s_0): the state changes by rounding-level
  amounts only (|s| < 1e-13 s_0 in the dropped directions) and every bond
  stays full rank.

Pins: ``tests/test_adjoint_oracle.py`` checks the SVD adjoint against central
finite differences on random matrices, the untruncated MPDO gradient against
autograd through the exact dense density-matrix simulator, and the truncated
MPDO gradient against complex128 central finite differences (h = 1e-4) of the
same evolution.
"""
from __future__ import annotations

import math
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np
import torch

from . import mpdo_oracle as O

# relative broadening of the 1/(s_j^2 - s_i^2) terms: eta = (BROADENING s_0^2)^2
BROADENING = 1e-12
# singular values below RANK_TOL * s_0 are dropped from differentiated splits
RANK_TOL = 1e-13


def _inv(s: torch.Tensor) -> torch.Tensor:
    return torch.where(s > 0, 1 / torch.where(s > 0, s, torch.ones_like(s)), torch.zeros_like(s))


class _TruncatedSVD(torch.autograd.Function):
    """(u_k, s_k, vh_k, s_rest) = truncated thin SVD of a matrix."""

    @staticmethod
    def forward(ctx, M, max_sv, max_err, relative, broadening):
        dt = M.dtype
        u, s, vh = O._svd128(M.detach().to(torch.complex128))
        k = O.keep_count(s, max_sv, max_err, relative)
        if RANK_TOL > 0 and k > 1:
            # numerical rank: singular values at the rounding level of s_0 are
            # zeros of the exact factorisation; keeping them (the chi cap
            # does whenever it exceeds the rank) would hand the next QR a
            # singular R, where its adjoint is undefined
            k = max(1, min(k, int((s > RANK_TOL * s[0]).sum())))
        ctx.save_for_backward(u, s, vh)
        ctx.k, ctx.dt, ctx.broadening = k, dt, broadening
        rdt = torch.float64 if dt == torch.complex128 else torch.float32
        return (u[:, :k].to(dt).clone(), s[:k].to(rdt).clone(), vh[:k].to(dt).clone(), s[k:].to(rdt).clone())

    @staticmethod
    def backward(ctx, gu, gs, gvh, _g_rest):
        u, s, vh = ctx.saved_tensors
        k = ctx.k
        m, p, n = u.shape[0], s.numel(), vh.shape[1]
        c = torch.complex128
        GU = torch.zeros(m, p, dtype=c)
        GS = torch.zeros(p, dtype=torch.float64)
        GV = torch.zeros(n, p, dtype=c)
        if gu is not None:
            GU[:, :k] = gu.to(c)
        if gs is not None:
            GS[:k] = gs.to(torch.float64)
        if gvh is not None:
            GV[:, :k] = gvh.to(c).conj().T
        v = vh.conj().T
        J = u.conj().T @ GU                                   # U^H dL/dU
        Mv = v.conj().T @ GV                                  # V^H dL/dV
        s2 = s * s
        D = s2[None, :] - s2[:, None]                         # D_ij = s_j^2 - s_i^2
        eta = (ctx.broadening * (s2[0] if p else 0.0)) ** 2
        F = D / (D * D + eta) if eta > 0 else torch.where(D != 0, 1 / torch.where(D != 0, D, 1), 0)
        F.fill_diagonal_(0)
        sc, si = s.to(c), _inv(s).to(c)
        K = (F * (J - J.conj().T)) * sc[None, :] + sc[:, None] * (F * (Mv - Mv.conj().T))
        K = K + torch.diag(GS.to(c) + 1j * J.diagonal().imag * _inv(s))
        GA = u @ K @ vh
        GA = GA + ((GU - u @ J) * si[None, :]) @ vh           # (I - U U^H) G_U S^-1 V^H
        GA = GA + (u * si[None, :]) @ (GV - v @ Mv).conj().T  # U S^-1 G_V^H (I - V V^H)
        return GA.to(ctx.dt), None, None, None, None


def truncated_svd(M: torch.Tensor, max_singular_values: Optional[int] = None,
                  max_truncation_error: Optional[float] = None, relative: bool = False,
                  broadening: float = BROADENING):
    """``mpdo_oracle.svd_truncate`` (decompositions.py:108-146, exact SVD)
    with the broadened SVD adjoint as its backward."""
    return _TruncatedSVD.apply(M, max_singular_values, max_truncation_error, relative, broadening)


# ----------------------------------------------------------------------------
# differentiable gates and channels (same matrices as mpdo_oracle.gate_1q,
# gate_2q and depolarization)
# ----------------------------------------------------------------------------
def _cplx(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.float64).to(torch.complex128)


def ry(theta: torch.Tensor) -> torch.Tensor:
    """YGates.py:65-67."""
    c, s = _cplx(torch.cos(theta / 2)), _cplx(torch.sin(theta / 2))
    return torch.stack([torch.stack([c, -s]), torch.stack([s, c])])


def rz(theta: torch.Tensor) -> torch.Tensor:
    """ZGates.py:65-66."""
    e = torch.exp(-0.5j * _cplx(theta))
    z = torch.zeros((), dtype=torch.complex128)
    return torch.stack([torch.stack([e, z]), torch.stack([z, e.conj()])])


def rx(theta: torch.Tensor) -> torch.Tensor:
    """XGates.py:65-67."""
    c, s = _cplx(torch.cos(theta / 2)), _cplx(torch.sin(theta / 2))
    return torch.stack([torch.stack([c, -1j * s]), torch.stack([-1j * s, c])])


def u3(theta: torch.Tensor, phi: torch.Tensor, lam: torch.Tensor) -> torch.Tensor:
    """SingleGates.py:179-185."""
    c, s = _cplx(torch.cos(theta / 2)), _cplx(torch.sin(theta / 2))
    el, ep = torch.exp(1j * _cplx(lam)), torch.exp(1j * _cplx(phi))
    return torch.stack([torch.stack([c, -el * s]), torch.stack([ep * s, el * ep * c])])


_PAULI_T = torch.as_tensor(np.stack(O._PAULI).astype(np.complex128))


def depolarization(p: torch.Tensor, qn: int = 1) -> torch.Tensor:
    """NoiseChannel.py:51-91 with a differentiable probability: Kraus weights
    sqrt(1 - (4^n - 1) p / 4^n) on the identity string and sqrt(p / 4^n) on
    the others, layout [out..., in..., k]."""
    d = 4 ** qn
    p = p.to(torch.float64)
    w = torch.cat([torch.sqrt(1 - (d - 1) * p / d).reshape(1), torch.sqrt(p / d).expand(d - 1)])
    ops = _PAULI_T
    for _ in range(qn - 1):
        ops = torch.stack([torch.kron(e, b) for e in ops for b in _PAULI_T])
    t = ops * _cplx(w)[:, None, None]                          # [k, f, f']
    return t.permute(1, 2, 0).reshape([2] * (2 * qn) + [d])


def noisy_1q(g: torch.Tensor, p: Optional[torch.Tensor]) -> torch.Tensor:
    """Depolarising after the gate (Circuit.py:146-155 with the decay slot the
    identity): [out, in, k]."""
    if p is None:
        return g
    return torch.einsum('xyk,ys->xsk', depolarization(p, 1), g)


def noisy_2q(g: torch.Tensor, p: Optional[torch.Tensor]) -> torch.Tensor:
    """Circuit.py:95: einsum('ijklp, klmn -> ijmnp'), 2q depolarising after the gate."""
    if p is None:
        return g
    return torch.einsum('ijklp,klmn->ijmnp', depolarization(p, 2), g)


_CZ = O.gate_2q('CZ')


# ----------------------------------------------------------------------------
# the gradient workload: hardware-efficient ansatz with trainable noise
# ----------------------------------------------------------------------------
def ansatz_angles(n: int, layers: int, seed: int = 0) -> torch.Tensor:
    """Angles [layers, 2, n] (RY then RZ per qubit) ~ U[0, 2pi) from
    ``torch.Generator().manual_seed(seed)``."""
    g = torch.Generator().manual_seed(seed)
    return 2 * math.pi * torch.rand(layers, 2, n, dtype=torch.float64, generator=g)


def ansatz_ops(angles: torch.Tensor, p: Optional[Dict[str, torch.Tensor]] = None) -> list:
    """Op list (``mpdo_oracle.evolve`` format) of the hardware-efficient
    ansatz: per layer an RY sublayer, an RZ sublayer and a CZ ladder
    (0,1), (1,2), ..., (n-2,n-1), each sublayer followed by a truncate.
    ``p`` = {'ry': p, 'rz': p, 'cz': p} depolarising probabilities (one per
    gate type) or None for a noiseless circuit."""
    layers, _, n = angles.shape
    p = p or {}
    ops = []
    for l in range(layers):
        for j, (gate, key) in enumerate(((ry, 'ry'), (rz, 'rz'))):
            ops += [('1q', q, noisy_1q(gate(angles[l, j, q]), p.get(key))) for q in range(n)]
            ops.append(('truncate',))
        cz = noisy_2q(_CZ, p.get('cz'))
        ops += [('2q', q, q + 1, cz) for q in range(n - 1)]
        ops.append(('truncate',))
    return ops


_Z = torch.as_tensor(O._PAULI[3].astype(np.complex128))
_X = torch.as_tensor(O._PAULI[1].astype(np.complex128))


def ising_energy(st: O.MPDO, hx: float = 0.5) -> torch.Tensor:
    """sum_i <Z_i Z_{i+1}> + hx sum_i <X_i> (unnormalised Tr(rho O), as
    dmOperations.pauli_expect returns)."""
    e = sum(O.expect_ops(st, {i: _Z, i + 1: _Z}) for i in range(st.n - 1))
    return e + hx * sum(O.expect_ops(st, {i: _X}) for i in range(st.n))


def ising_energy_dense(rho: torch.Tensor, n: int, hx: float = 0.5) -> torch.Tensor:
    """The same observable on a dense 2^n x 2^n density matrix (qubit 0 most
    significant)."""
    def op(ops: Dict[int, torch.Tensor]):
        m = torch.ones(1, 1, dtype=torch.complex128)
        for q in range(n):
            m = torch.kron(m, ops.get(q, torch.eye(2, dtype=torch.complex128)))
        return m
    obs = sum(op({i: _Z, i + 1: _Z}) for i in range(n - 1)) + hx * sum(op({i: _X}) for i in range(n))
    return torch.trace(rho @ obs).real


def energy(angles: torch.Tensor, p: Optional[Dict[str, torch.Tensor]], chi: Optional[int],
           kappa: Optional[int], hx: float = 0.5) -> torch.Tensor:
    """Loss of the gradient workload: evolve |0...0> (connected chain) through
    the ansatz with the reference's truncation placement and return the Ising
    energy."""
    n = angles.shape[2]
    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, ansatz_ops(angles, p), chi=chi, kappa=kappa, noisy=p is not None)
    return ising_energy(st, hx)


def central_fd(f: Callable[[], torch.Tensor], params: Sequence[torch.Tensor], h: float = 1e-4) -> List[torch.Tensor]:
    """Central finite differences (f(x + h) - f(x - h)) / 2h of a scalar
    function of real parameter tensors, each entry perturbed in place."""
    out = []
    with torch.no_grad():
        for x in params:
            g = torch.zeros_like(x)
            flat, gflat = x.view(-1), g.view(-1)
            for i in range(flat.numel()):
                x0 = flat[i].item()
                flat[i] = x0 + h
                fp = float(f())
                flat[i] = x0 - h
                fm = float(f())
                flat[i] = x0
                gflat[i] = (fp - fm) / (2 * h)
            out.append(g)
    return out
