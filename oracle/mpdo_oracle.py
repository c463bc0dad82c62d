"""Plain-torch CPU restatement of the reference MPDO evolution path.

TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the product
never imports it.

Site tensors use one fixed layout, ``A[l, s, a, r]``:
  l = left bond, s = physical (2), a = inner / Kraus leg ``I_k``, r = right bond.
A site that never received a Kraus leg has ``a == 1``, which is equivalent to the
reference's missing ``I_k`` edge for every operation below.

Every function cites the reference lines it restates (paths relative to the
reference project root).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

# Circuit.py:22-23
GLOBAL_MINIMUM = 2.718281828459045 * 1e-8
MAX_ATTEMPTS = 4

# decompositions.py:112 -- randomized SVD switch of the vendored backend patch
RANDOMIZED_MIN_NUMEL = 10000


# ----------------------------------------------------------------------------
# gate matrices (QuantumGates/*.py).  Index order [out, in]; 2q gates are
# reshaped to [out0, out1, in0, in1] (DoubleGates.py:29-31 and siblings).
# ----------------------------------------------------------------------------
def _c(x, dtype):
    return torch.as_tensor(x, dtype=dtype)


def gate_1q(name: str, *p, dtype=torch.complex128) -> torch.Tensor:
    """Single-qubit gate matrices (SingleGates.py, XGates.py, YGates.py,
    ZGates.py, PhaseGates.py)."""
    j = 1j
    name = name.upper()
    if name in ('I', 'MEASUREZ'):
        m = [[1, 0], [0, 1]]                                   # SingleGates.py:31, 318
    elif name in ('H', 'MEASUREX'):
        s = 1 / math.sqrt(2)
        m = [[s, s], [s, -s]]                                  # SingleGates.py:64, 247
    elif name == 'MEASUREY':
        s = 1 / math.sqrt(2)
        m = [[s, -j * s], [s, j * s]]                          # SingleGates.py:281
    elif name == 'X':
        m = [[0, 1], [1, 0]]                                   # XGates.py:29
    elif name == 'Y':
        m = [[0, -j], [j, 0]]                                  # YGates.py:29
    elif name == 'Z':
        m = [[1, 0], [0, -1]]                                  # ZGates.py:29
    elif name == 'S':
        m = [[1, 0], [0, j]]                                   # PhaseGates.py:30
    elif name == 'SDG':
        m = [[1, 0], [0, -j]]                                  # PhaseGates.py:63
    elif name == 'T':
        m = [[1, 0], [0, (1 + j) / math.sqrt(2)]]              # PhaseGates.py:96
    elif name == 'RX':
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        m = [[c, -j * s], [-j * s, c]]                         # XGates.py:65-67
    elif name == 'RY':
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        m = [[c, -s], [s, c]]                                  # YGates.py:65-67
    elif name == 'RZ':
        m = [[np.exp(-j * p[0] / 2), 0], [0, np.exp(j * p[0] / 2)]]   # ZGates.py:65-66
    elif name in ('P', 'U1'):
        m = [[1, 0], [0, np.exp(j * p[0])]]                    # PhaseGates.py:132, SingleGates.py:100
    elif name == 'U2':
        # SingleGates.py:139-143 (the reference reads an undefined attribute
        # there; this is the evident intent)
        lm, pm = np.exp(j * p[1]), np.exp(j * p[0])
        s = 1 / math.sqrt(2)
        m = [[s, -lm * s], [pm * s, lm * pm * s]]
    elif name == 'U3':
        th, ph, lam = p
        lm, pm = np.exp(j * lam), np.exp(j * ph)
        c, s = math.cos(th / 2), math.sin(th / 2)
        m = [[c, -lm * s], [pm * s, lm * pm * c]]              # SingleGates.py:179-185
    elif name == 'RESET0':
        m = [[1, 0], [0, 0]]                                   # SingleGates.py:350
    elif name == 'RESET1':
        m = [[0, 0], [0, 1]]                                   # SingleGates.py:384
    else:
        raise ValueError(f'unknown 1q gate {name}')
    return _c(m, dtype)


def gate_2q(name: str, *p, dtype=torch.complex128) -> torch.Tensor:
    """Two-qubit gate tensors [o0, o1, i0, i1] (DoubleGates.py, XGates.py,
    YGates.py, ZGates.py, PhaseGates.py)."""
    j = 1j
    name = name.upper()
    if name == 'II':
        m = np.eye(4)                                          # DoubleGates.py:29-31
    elif name in ('CX', 'CNOT'):
        m = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]   # XGates.py:102-104
    elif name == 'CY':
        m = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -j], [0, 0, j, 0]]  # YGates.py:102-105
    elif name == 'CZ':
        m = np.diag([1, 1, 1, -1])                             # ZGates.py:101-103
    elif name == 'SWAP':
        m = [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]]   # DoubleGates.py:134-136
    elif name == 'ISWAP':
        m = [[1, 0, 0, 0], [0, 0, j, 0], [0, j, 0, 0], [0, 0, 0, 1]]   # DoubleGates.py:99-101
    elif name == 'PSWAP':
        c, s = math.cos(p[0]), math.sin(p[0])
        m = [[1, 0, 0, 0], [0, c, s, 0], [0, s, c, 0], [0, 0, 0, 1]]   # DoubleGates.py:171-174
    elif name == 'CP':
        m = np.diag([1, 1, 1, np.exp(j * p[0])])               # PhaseGates.py:171-174
    elif name == 'RXX':
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        m = [[c, 0, 0, -j * s], [0, c, -j * s, 0], [0, -j * s, c, 0], [-j * s, 0, 0, c]]  # XGates.py:140-144
    elif name == 'RYY':
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        m = [[c, 0, 0, -s], [0, c, s, 0], [0, -s, c, 0], [s, 0, 0, c]]  # YGates.py:141-145
    elif name == 'RZZ':
        mi, pl = np.exp(-j * p[0] / 2), np.exp(j * p[0] / 2)
        m = np.diag([mi, pl, pl, mi])                          # ZGates.py:139-143
    elif name == 'XXPLUSYY':
        th, beta = p
        c, s = math.cos(th / 2), -j * math.sin(th / 2)
        m = [[1, 0, 0, 0], [0, c, s * np.exp(j * beta), 0],
             [0, s * np.exp(-j * beta), c, 0], [0, 0, 0, 1]]   # DoubleGates.py:247-254
    else:
        raise ValueError(f'unknown 2q gate {name}')
    return _c(np.asarray(m, dtype=np.complex128), dtype).reshape(2, 2, 2, 2)


# ----------------------------------------------------------------------------
# noise channels (NoiseChannel.py, ChipInfo.py).  Kraus tensors carry the Kraus
# index last: (2, 2, K) = [out, in, k]; (2, 2, 2, 2, K) = [o0, o1, i0, i1, k].
# ----------------------------------------------------------------------------
_PAULI = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]),
          np.array([[1, 0], [0, -1]])]                         # NoiseChannel.py:34-37


def depolarization(p: float, qn: int = 1, dtype=torch.complex128) -> torch.Tensor:
    """NoiseChannel.py:51-91: weights sqrt(1-(4^n-1)p/4^n), sqrt(p/4^n); Pauli
    strings in kron order with the first qubit slowest (82-88); layout via
    einsum('ij,jfk->fki') then reshape to [out..., in..., k] (89-90)."""
    if not 0 <= p <= 1:
        raise ValueError('Probability p must be in the range [0, 1].')
    d = 4 ** qn
    w = [math.sqrt(1 - (d - 1) * p / d)] + [math.sqrt(p / d)] * (d - 1)
    ops = list(_PAULI)
    for _ in range(qn - 1):
        ops = [np.kron(e, b) for e in ops for b in _PAULI]
    t = np.stack(ops) * np.asarray(w)[:, None, None]          # [k, f, k']
    t = np.transpose(t, (1, 2, 0)).reshape([2] * (2 * qn) + [d])
    return torch.as_tensor(t.astype(np.complex128), dtype=dtype)


def amplitude_damping(gamma: float, dtype=torch.complex128) -> torch.Tensor:
    """Decay Kraus pair with damping parameter ``gamma`` (NoiseChannel.py:149-155)."""
    k = np.array([[[1, 0], [0, math.sqrt(1 - gamma)]],
                  [[0, math.sqrt(gamma)], [0, 0]]], dtype=np.complex128)
    return torch.as_tensor(np.transpose(k, (1, 2, 0)), dtype=dtype)


def decay(bath_rate: float, gamma: float, gate_time: float, dtype=torch.complex128):
    """NoiseChannel.py:144-155."""
    if gate_time <= 0:
        raise ValueError('The gate time must be greater than 0, or set the gate to IDEAL.')
    return amplitude_damping(1 - math.exp(-bath_rate * gamma * gate_time), dtype)


def dephasing(bath_rate: float, gamma: float, gate_time: float, dtype=torch.complex128):
    """NoiseChannel.py:157-170."""
    if gate_time <= 0:
        raise ValueError('The gate time must be greater than 0, or set the gate to IDEAL.')
    p = 1 - math.exp(-bath_rate * gamma * gate_time)
    sp, s1 = math.sqrt(p), math.sqrt(1 - p)
    k = np.array([[[s1, 0], [0, s1]], [[sp, 0], [0, 0]], [[0, 0], [0, sp]]], dtype=np.complex128)
    return torch.as_tensor(np.transpose(k, (1, 2, 0)), dtype=dtype)


def amp_phase_damping(time: float, T1: float, T2: float, dtype=torch.complex128):
    """NoiseChannel.py:93-142."""
    if time < 0 or T1 <= 0 or T2 <= 0:
        raise ValueError('The time, T1, T2 must be greater than or equal to 0')
    t2p = 2 * T1 * T2 / (2 * T1 - T2)
    p1 = 1 - math.exp(-time / T1)
    p2 = 1 - math.exp(-time / t2p)
    k = np.array([[[1, 0], [0, math.sqrt(1 - (p1 + p2))]],
                  [[0, 0], [0, math.sqrt(p2)]],
                  [[0, math.sqrt(p1)], [0, 0]]], dtype=np.complex128)
    return torch.as_tensor(np.transpose(k, (1, 2, 0)), dtype=dtype)


CHIPS = {  # ChipInfo.py:44-87 (gate_time, bath_rate, decay_rate, dephasing_rate, T1, T2, dpc)
    'best': (30, 0., 0.0, 0.0, 2e11, 2e10, 11e-4),
    'medium': (1, 0.01, 0.98, 0.02, 2e11, 2e10, 5e-2),
    'worst': (30, 0., 0.0, 0.0, 2e2, 2e1, 11e-2),
}


def chip_channels(chip: Optional[str] = None, dtype=torch.complex128):
    """NoiseChannel.__init__ (NoiseChannel.py:20-46) for a named chip preset."""
    gt, bath, dec, dep, T1, T2, dpc = CHIPS[chip or 'worst']
    return dict(decay=decay(bath, dec, gt, dtype), dephasing=dephasing(bath, dep, gt, dtype),
                dpc=depolarization(dpc, 1, dtype), dpc2=depolarization(dpc, 2, dtype),
                apde=amp_phase_damping(gt, T1, T2, dtype))


def noisy_1q(decay_t: torch.Tensor, dephasing_t: torch.Tensor, g: torch.Tensor) -> torch.Tensor:
    """Circuit.py:146-155: einsum('nlm, ljk, ji -> nimk').reshape(2, 2, -1) -- the
    dephasing slot acts after the gate, then the decay slot; Kraus index
    (m_decay, k_dephasing) row-major."""
    return torch.einsum('nlm,ljk,ji->nimk', decay_t, dephasing_t, g).reshape(2, 2, -1)


def noisy_2q(dpc2: torch.Tensor, g: torch.Tensor) -> torch.Tensor:
    """Circuit.py:95: einsum('ijklp, klmn -> ijmnp') -- 2q depolarising after the gate."""
    return torch.einsum('ijklp,klmn->ijmnp', dpc2, g)


# ----------------------------------------------------------------------------
# chi-matrix -> Kraus (RealNoise.py, Tools.py:466-509)
# ----------------------------------------------------------------------------
def _name2matrix(name: str) -> np.ndarray:
    """Tools.py:488-509 with Y~ = -iY (Tools.py:504), kron order (508-509)."""
    ops = {'I': np.eye(2), 'X': np.array([[0, 1], [1, 0]]),
           'Y': -1j * np.array([[0, -1j], [1j, 0]]), 'Z': np.array([[1, 0], [0, -1]])}
    out = np.array([[1.0 + 0j]])
    for ch in name:
        out = np.kron(out, ops[ch])
    return out


def chi_to_kraus(chi: np.ndarray, dtype=torch.complex128) -> torch.Tensor:
    """RealNoise.py:35-170: eig of the process matrix, descending complex
    argsort (76-79), count of |lambda| > 1e-12 (92-94), sqrt(lambda)-scaled
    eigenvectors with entries below 1e-12 zeroed (96-102), Kraus operator
    sum_j e_j P_j over Pauli strings, reshape (2,2,2,2) and stack with the
    Kraus index last (168-169)."""
    import itertools
    s, u = np.linalg.eig(chi)
    idx = s.argsort()[::-1]
    s, u = s[idx], u[:, idx]
    count = int(np.sum(np.abs(s) > 1e-12))
    nq = int(round(math.log(chi.shape[0], 4)))
    names = [''.join(g) for g in itertools.product('IXYZ', repeat=nq)]
    kraus = []
    for i in range(count):
        e = u[:, i] * np.sqrt(s[i] + 0j)
        e = np.where(np.abs(e) < 1e-12, 0, e)
        op = sum(e[jj] * _name2matrix(names[jj]) for jj in range(len(names)))
        kraus.append(op.reshape([2] * (2 * nq)))
    t = np.stack(kraus)                                      # [k, o0, o1, i0, i1]
    t = np.moveaxis(t, 0, -1)                                 # einsum('ijlmn->jlmni')
    return torch.as_tensor(t.astype(np.complex128), dtype=dtype)


def read_chi(filename: str) -> np.ndarray:
    """RealNoise.py:22-32."""
    if '.mat' in filename:
        from scipy.io import loadmat
        return loadmat(filename)['exp']
    if '.npz' in filename:
        return np.load(filename)['chi']
    raise TypeError('Current file-type is not supported.')


# ----------------------------------------------------------------------------
# decompositions (decompositions.py:23-195, the vendored backend patch)
# ----------------------------------------------------------------------------
def randomized_svd(M: torch.Tensor, n_components: int, n_oversamples: int = 7):
    """decompositions.py:23-48: fresh CPU generator at its default seed every
    call, 3 (m >= n) or 2 power iterations, QR, SVD of the projection."""
    m, n = M.shape
    rng = torch.Generator()
    q = torch.randn(m, n_components + n_oversamples, dtype=torch.complex64, generator=rng)
    q = q.to(M.dtype)
    n_iter = 3 if m >= n else 2
    for _ in range(n_iter):
        q = M @ (M.conj().T @ q)
    q, _ = _qr(q)
    b = q.conj().T @ M
    u, s, vh = _svd(b)
    return q @ u, s, vh


_AARCH64 = __import__('platform').machine() in ('aarch64', 'arm64')


def _svd128(M: torch.Tensor):
    if _AARCH64:
        # the divide-and-conquer SVD of the Arm hosts' LAPACK aborts the whole
        # process (xerbla) on some inputs; the QR-iteration driver does not
        import scipy.linalg
        u, s, vh = scipy.linalg.svd(M.numpy(), full_matrices=False, lapack_driver='gesvd')
        return torch.from_numpy(u), torch.from_numpy(s), torch.from_numpy(vh)
    return torch.linalg.svd(M, full_matrices=False)


def _svd(M: torch.Tensor):
    """Thin SVD.  complex64 inputs are factorised in complex128 and the factors
    rounded back to complex64 (the state keeps fp32 storage)."""
    if M.dtype == torch.complex64:
        u, s, vh = _svd128(M.to(torch.complex128))
        return u.to(torch.complex64), s.to(torch.float32), vh.to(torch.complex64)
    return _svd128(M)


def _qr(M: torch.Tensor):
    if M.dtype == torch.complex64:
        q, r = torch.linalg.qr(M.to(torch.complex128))
        return q.to(torch.complex64), r.to(torch.complex64)
    return torch.linalg.qr(M)


def svd_truncate(M: torch.Tensor, max_singular_values: Optional[int] = None,
                 max_truncation_error: Optional[float] = None, relative: bool = False,
                 randomized: bool = False):
    """decompositions.py:108-146 on a matrix: returns (u, s, vh, s_rest).

    The error rule is the patch's: keep ``idx + 1`` singular values at the first
    ``idx`` where ``sqrt(cumsum(s^2))[-1] - sqrt(cumsum(s^2))[idx] <= err`` (121-132).
    ``randomized`` reproduces the patch's switch to the randomized SVD for
    matrices with >= 10000 elements and a singular-value cap (112-115); it is
    off by default (exact SVD).

    A complex128 ``M`` that requires grad goes through the gradient oracle's
    truncated SVD (``oracle.adjoint``): the same factors and keep rule, with a
    backward of its own."""
    if M.requires_grad and torch.is_grad_enabled() and not randomized:
        from .adjoint import truncated_svd
        return truncated_svd(M, max_singular_values, max_truncation_error, relative)
    if randomized and M.numel() >= RANDOMIZED_MIN_NUMEL and max_singular_values is not None:
        u, s, vh = randomized_svd(M, max_singular_values)
    else:
        u, s, vh = _svd(M)
    keep = keep_count(s, max_singular_values, max_truncation_error, relative)
    return u[:, :keep], s[:keep], vh[:keep, :], s[keep:]


def keep_count(s: torch.Tensor, max_singular_values: Optional[int], max_truncation_error: Optional[float],
               relative: bool) -> int:
    """decompositions.py:121-140: how many of the descending singular values
    ``s`` a split keeps."""
    if max_singular_values is None:
        max_singular_values = s.numel()
    n_err = max_singular_values
    if max_truncation_error is not None:
        te = torch.sqrt(torch.cumsum(s ** 2, dim=0))
        thr = max_truncation_error * s[0] if relative else max_truncation_error
        for idx in range(te.shape[0] - 1):
            if te[-1] - te[idx] <= thr:
                n_err = idx + 1
                break
    return min(max_singular_values, n_err)


# ----------------------------------------------------------------------------
# MPDO state and the hot-path operations
# ----------------------------------------------------------------------------
@dataclass
class MPDO:
    sites: List[torch.Tensor]                 # A[l, s, a, r]
    bonds: List[bool]                         # bond (k, k+1) exists (tn edge present)
    discarded: List[float] = field(default_factory=list)   # per-bond weight of the last sweep

    @property
    def n(self):
        return len(self.sites)

    def clone(self) -> 'MPDO':
        return MPDO([s.clone() for s in self.sites], list(self.bonds), list(self.discarded))

    def dims(self):
        return [tuple(s.shape) for s in self.sites]


def product_state(vectors: Sequence[Sequence[complex]], connected: bool = False,
                  dtype=torch.complex128) -> MPDO:
    """Tools.py:110-198 (create_ket*Series): one node per qubit with only a
    physical leg.  ``connected=True`` adds dimension-1 bonds between neighbours,
    which the reference accepts as an input state and which makes
    ``checkConnectivity`` (TNNOptimizer.py:51-61) true from the start."""
    sites = [torch.as_tensor(np.asarray(v, dtype=np.complex128), dtype=dtype).reshape(1, 2, 1, 1)
             for v in vectors]
    return MPDO(sites, [connected] * (len(sites) - 1))


def apply_1q(st: MPDO, site: int, g: torch.Tensor) -> None:
    """Circuit.py:138-178: contract the gate's inner leg with ``physics_k``; a
    Kraus leg is flattened into ``I_k`` with the old leg first (174-178)."""
    a = st.sites[site]
    if g.dim() == 2:
        g = g.unsqueeze(-1)
    K = g.shape[-1]
    l, _, aa, r = a.shape
    out = torch.einsum('xsk,lsar->lxakr', g.to(a.dtype), a)
    st.sites[site] = out.reshape(l, 2, aa * K, r)


def _split_theta(st: MPDO, i: int, theta: torch.Tensor, cutoff: float) -> None:
    l, x, aa, y, cc, r = theta.shape
    m = theta.reshape(l * x * aa, y * cc * r)
    for attempt in range(MAX_ATTEMPTS):                       # Circuit.py:118-136
        try:
            u, s, vh, _ = svd_truncate(m, None, cutoff, relative=False)
            break
        except torch.linalg.LinAlgError:
            nrm = torch.linalg.norm(m).item()
            mag = torch.finfo(torch.float64).eps * max(nrm, 1.0) * GLOBAL_MINIMUM * 1e-2
            m = m + mag * (torch.randn_like(m.real) + 1j * torch.randn_like(m.real)).to(m.dtype)
    else:
        raise torch.linalg.LinAlgError('SVD failed after perturbation retries')
    ss = torch.sqrt(s).to(m.dtype)                           # tn.split_node: sqrt(S) on both factors
    k = s.numel()
    st.sites[i] = (u * ss[None, :]).reshape(l, x, aa, k)
    st.sites[i + 1] = (ss[:, None] * vh).reshape(k, y, cc, r)


def apply_2q(st: MPDO, i: int, t: torch.Tensor, cutoff: float = GLOBAL_MINIMUM) -> None:
    """Circuit.py:74-136 for the nearest-neighbour pair (i, i+1).

    ``t`` is [o_i, o_{i+1}, in_i, in_{i+1}] or with a trailing Kraus leg.  The
    two sites are contracted over their shared bond (contractors.optimal,
    104-107), the gate is applied, the Kraus leg is flattened into
    ``I_{i+1}`` after the old one (109-114), and the block is split by an exact
    SVD with absolute cutoff ``GLOBAL_MINIMUM`` and sqrt(S) on both sides
    (116-126)."""
    a, b = st.sites[i], st.sites[i + 1]
    if t.dim() == 4:
        t = t.unsqueeze(-1)
    t = t.to(a.dtype)
    theta = torch.einsum('lsam,mtcr->lsatcr', a, b)
    theta = torch.einsum('xystk,lsatcr->lxaycrk', t, theta)
    l, x, aa, y, cc, r, K = theta.shape
    theta = theta.permute(0, 1, 2, 3, 4, 6, 5).reshape(l, x, aa, y, cc * K, r)
    _split_theta(st, i, theta, cutoff)
    st.bonds[i] = True


def connected(st: MPDO) -> bool:
    """TNNOptimizer.py:51-61 (tn.check_connected on the chain)."""
    return st.n <= 1 or all(st.bonds)


def qr_left2right(st: MPDO) -> None:
    """TNNOptimizer.py:87-108: reduced QR of (all legs but the right bond) x
    (right bond) per site; R absorbed into the next site."""
    for i in range(st.n - 1):
        l, x, aa, r = st.sites[i].shape
        q, rr = _qr(st.sites[i].reshape(l * x * aa, r))
        k = q.shape[1]
        st.sites[i] = q.reshape(l, x, aa, k)
        st.sites[i + 1] = torch.einsum('kr,rsac->ksac', rr, st.sites[i + 1])


def svd_right2left(st: MPDO, chi: Optional[int], max_err: Optional[float],
                   randomized: bool = False) -> List[float]:
    """TNNOptimizer.py:111-134: contract sites (idx-1, idx), SVD keeping <= chi
    (relative error rule), sqrt(S) on both sides.  Returns the discarded weight
    sum(s_rest^2)/sum(s^2) per bond (the values the reference drops at 129)."""
    disc = [0.0] * (st.n - 1)
    for idx in range(st.n - 1, 0, -1):
        a, b = st.sites[idx - 1], st.sites[idx]
        l, x, aa, _ = a.shape
        _, y, cc, r = b.shape
        m = torch.einsum('lsam,mtcr->lsatcr', a, b).reshape(l * x * aa, y * cc * r)
        u, s, vh, rest = svd_truncate(m, chi, max_err, relative=True, randomized=randomized)
        tot = float((s.detach() ** 2).sum() + (rest.detach() ** 2).sum())
        disc[idx - 1] = float((rest.detach() ** 2).sum()) / tot if tot > 0 else 0.0
        ss = torch.sqrt(s).to(m.dtype)
        k = s.numel()
        st.sites[idx - 1] = (u * ss[None, :]).reshape(l, x, aa, k)
        st.sites[idx] = (ss[:, None] * vh).reshape(k, y, cc, r)
    st.discarded = disc
    return disc


def svd_left2right(st: MPDO, chi: Optional[int], max_err: Optional[float]) -> List[float]:
    """TNNOptimizer.py:137-161: the mirror sweep, pairs (idx, idx+1) for idx =
    0 .. n-2, the same split (<= chi, relative error rule, sqrt(S) on both
    sides).  Returns the discarded weight per bond."""
    disc = [0.0] * (st.n - 1)
    for idx in range(st.n - 1):
        a, b = st.sites[idx], st.sites[idx + 1]
        l, x, aa, _ = a.shape
        _, y, cc, r = b.shape
        m = torch.einsum('lsam,mtcr->lsatcr', a, b).reshape(l * x * aa, y * cc * r)
        u, s, vh, rest = svd_truncate(m, chi, max_err, relative=True)
        tot = float((s ** 2).sum() + (rest ** 2).sum())
        disc[idx] = float((rest ** 2).sum()) / tot if tot > 0 else 0.0
        ss = torch.sqrt(s).to(m.dtype)
        k = s.numel()
        st.sites[idx] = (u * ss[None, :]).reshape(l, x, aa, k)
        st.sites[idx + 1] = (ss[:, None] * vh).reshape(k, y, cc, r)
    st.discarded = disc
    return disc


def svd_kappa(st: MPDO, kappa: Optional[int], max_err: Optional[float],
              randomized: bool = False) -> None:
    """TNNOptimizer.py:164-197: per site with dim(I_k) > kappa, SVD of
    (other legs) x (I_k) keeping kappa; the site becomes U.S (V dropped)."""
    if kappa is None and max_err is None:
        return
    for i in range(st.n):
        l, x, aa, r = st.sites[i].shape
        if aa == 1 or (kappa is not None and aa <= kappa):
            continue
        m = st.sites[i].permute(0, 1, 3, 2).reshape(l * x * r, aa)
        u, s, vh, _ = svd_truncate(m, kappa, max_err, relative=True, randomized=randomized)
        k = s.numel()
        us = u * s.to(m.dtype)[None, :]
        st.sites[i] = us.reshape(l, x, r, k).permute(0, 1, 3, 2).contiguous()


def truncate(st: MPDO, chi: Optional[int], kappa: Optional[int], max_err: Optional[float],
             noisy: bool, randomized: bool = False) -> None:
    """Circuit.py:476-481: connectivity guard, bondTruncate (TNNOptimizer.py:72-84),
    then the kappa pass for noisy circuits."""
    if not connected(st):
        return
    if chi is not None or max_err is not None:
        qr_left2right(st)
        svd_right2left(st, chi, max_err, randomized)
    if noisy:
        svd_kappa(st, kappa, max_err, randomized)


# ----------------------------------------------------------------------------
# circuits as op lists
#   ('1q', q, kraus)  kraus: (2,2) or (2,2,K)
#   ('2q', q0, q1, kraus)  kraus: (2,2,2,2) or (2,2,2,2,K), legs in (q0, q1) order
#   ('truncate',)  ('barrier',)
# ----------------------------------------------------------------------------
def orient_2q(q0: int, q1: int, t: torch.Tensor) -> Tuple[int, torch.Tensor]:
    """Reorder a 2q tensor given on (q0, q1) to (min, max) leg order."""
    if abs(q0 - q1) != 1:
        raise ValueError('only nearest-neighbour two-qubit gates are supported')
    if q0 < q1:
        return q0, t
    perm = [1, 0, 3, 2] + ([4] if t.dim() == 5 else [])
    return q1, t.permute(*perm)


def evolve(st: MPDO, ops, chi=None, kappa=None, max_err=None, noisy=False,
           randomized: bool = False, cutoff: float = GLOBAL_MINIMUM) -> MPDO:
    """Circuit.py:469-491.  ``cutoff`` is the split's absolute cutoff
    (GLOBAL_MINIMUM in the reference, Circuit.py:123)."""
    last = None
    for op in ops:
        kind = op[0]
        if kind == '1q':
            apply_1q(st, op[1], op[2])
        elif kind == '2q':
            i, t = orient_2q(op[1], op[2], op[3])
            apply_2q(st, i, t, cutoff)
        elif kind == 'truncate':
            truncate(st, chi, kappa, max_err, noisy, randomized)
        elif kind == 'barrier':
            pass
        else:
            raise ValueError(kind)
        last = kind
    if noisy and last != 'truncate' and last is not None:     # Circuit.py:487-489
        svd_kappa(st, kappa, max_err, randomized)
    return st


# ----------------------------------------------------------------------------
# readout (Circuit.py:226-295, dmOperations.py:18-201, Tools.py:242-273)
# ----------------------------------------------------------------------------
def _env_step(E: torch.Tensor, a: torch.Tensor, mode, op=None) -> torch.Tensor:
    """E[D, D', l, l'] -> E'[...] for one site.  mode: 'open', 'trace', 'op'."""
    D, Dp, l, lp = E.shape
    if mode == 'open':
        t = torch.einsum('DElm,lxar,myas->DxEyrs', E, a, a.conj())
        return t.reshape(D * 2, Dp * 2, a.shape[3], a.shape[3])
    if mode == 'trace':
        return torch.einsum('DElm,lxar,mxas->DErs', E, a, a.conj())
    return torch.einsum('DElm,lxar,yx,myas->DErs', E, a, op.to(a.dtype), a.conj())


def reduced_dm(st: MPDO, keep: Optional[Sequence[int]] = None) -> torch.Tensor:
    """Circuit.py:247-262 / 282-295: rho[(s_keep), (s'_keep)] with ket legs as
    rows and the Kraus legs traced (243).  ``keep`` defaults to all qubits."""
    keep = list(range(st.n)) if keep is None else sorted(keep)
    dt = st.sites[0].dtype
    E = torch.ones(1, 1, 1, 1, dtype=dt)
    for k, a in enumerate(st.sites):
        E = _env_step(E, a, 'open' if k in keep else 'trace')
    return E.reshape(E.shape[0], E.shape[1])


def expect_ops(st: MPDO, ops: dict) -> torch.Tensor:
    """Tr(rho . prod_k O_k) for single-site operators {site: O}; identity
    elsewhere (dmOperations.py:174-201 for Paulis).  Real part, unnormalised."""
    dt = st.sites[0].dtype
    E = torch.ones(1, 1, 1, 1, dtype=dt)
    for k, a in enumerate(st.sites):
        E = _env_step(E, a, 'op', ops[k]) if k in ops else _env_step(E, a, 'trace')
    return E.reshape(()).real


PAULI = {0: _PAULI[1], 1: _PAULI[2], 2: _PAULI[3]}            # dmOperations.py:11-15


def pauli_expect(st: MPDO, observables, oqs) -> torch.Tensor:
    """dmOperations.py:174-201."""
    observables = [observables] if isinstance(observables, int) else list(observables)
    oqs = [oqs] if isinstance(oqs, int) else list(oqs)
    ops = {q: torch.as_tensor(PAULI[o]) for o, q in zip(observables, oqs)}
    return expect_ops(st, ops)


def expect_dense(st: MPDO, obs: torch.Tensor, oq: Sequence[int]) -> torch.Tensor:
    """dmOperations.py:135-171 for one observable on qubits ``oq`` (matrix in
    the listed qubit order): Tr(rho_oq . O).real."""
    oq = list(oq)
    order = sorted(oq)
    rho = reduced_dm(st, order)
    m = len(oq)
    o = obs.reshape([2] * (2 * m)).to(rho.dtype)
    perm = [oq.index(q) for q in order] + [m + oq.index(q) for q in order]
    o = o.permute(*perm).reshape(2 ** m, 2 ** m)
    return torch.trace(rho @ o).real


_PROJ = [torch.tensor([[1, 0], [0, 0]], dtype=torch.complex128), torch.tensor([[0, 0], [0, 1]], dtype=torch.complex128)]


def trace_rho_rho(st0: MPDO, st1: MPDO, keep: Sequence[int]) -> float:
    """dmOperations.py:51-66: Tr(rho_0 rho_1) with both states traced over
    the qubits not in ``keep`` -- the doubled network contracted site by site
    (the reference lets tn.contractors.auto pick the order; the value does
    not depend on it): a kept qubit joins rho_0's ket with rho_1's bra and
    rho_0's bra with rho_1's ket, a traced one ket with bra in each state."""
    keep = set(int(q) for q in keep)
    E = torch.ones(1, 1, 1, 1, dtype=st0.sites[0].dtype)
    for k in range(st0.n):
        a0, a1 = st0.sites[k], st1.sites[k]
        if k in keep:
            E = torch.einsum('pqst,pxaP->qstxaP', E, a0)
            E = torch.einsum('qstxaP,qyaQ->stxyPQ', E, a0.conj())
            E = torch.einsum('stxyPQ,sybS->txPQbS', E, a1)
            E = torch.einsum('txPQbS,txbT->PQST', E, a1.conj())
        else:
            E = torch.einsum('pqst,pxaP->qstxaP', E, a0)
            E = torch.einsum('qstxaP,qxaQ->stPQ', E, a0.conj())
            E = torch.einsum('stPQ,szbS->tPQzbS', E, a1)
            E = torch.einsum('tPQzbS,tzbT->PQST', E, a1.conj())
    return float(E.reshape(()).real)


def conditional_p1(st: MPDO, order: Sequence[int], history: Sequence[int]) -> float:
    """Circuit.py:297-332: the probability that qubit ``order[len(history)]``
    reads 1 given that ``order[:len(history)]`` read ``history``, every other
    qubit traced: the two unnormalised outcome weights, each plus
    GLOBAL_MINIMUM, normalised.  The measurement basis is whatever ``st``
    holds (Circuit.py:413-418 rotates it first with MeasureX / MeasureY)."""
    q = order[len(history)]
    ops = {order[j]: _PROJ[h] for j, h in enumerate(history)}
    p = []
    for v in (0, 1):
        o = dict(ops)
        o[q] = _PROJ[v]
        p.append(float(expect_ops(st, o)) + GLOBAL_MINIMUM)
    if min(p) < 0:
        raise RuntimeError(f'State is illegal, and your probability distribution is {p}.')
    return p[1] / (p[0] + p[1])


def density2prob(rho: torch.Tensor) -> np.ndarray:
    """Tools.py:242-273 with _dict=False: |rho_ii| normalised by their sum."""
    p = torch.abs(torch.diagonal(rho)).double().numpy()
    return p / p.sum()


def trace(st: MPDO) -> float:
    """dmOperations.py:40-48."""
    return float(expect_ops(st, {}))


# ----------------------------------------------------------------------------
# timed CPU baseline: one layer of a circuit with a time budget
# ----------------------------------------------------------------------------
def time_layer(st: MPDO, layer_ops, chi, kappa, max_err=None, noisy=True, budget_s: float = 20.0,
               randomized: bool = False):
    """Run one layer (its gate sublayers and truncates) on the CPU and return
    the estimated wall time of the whole layer.  ``randomized`` takes the
    reference's randomized-SVD branch for capped SVDs of >= 10000 elements
    (decompositions.py:112-115), as its stock code path does.  Gate applications, QR sweeps
    and kappa passes run in full; SVD right-to-left sweeps run until the budget
    is spent and the remaining steps are extrapolated from the mean measured
    step time of the same bond kind (even / odd bond).  Returns
    (seconds, dict(measured=..., extrapolated_steps=...))."""
    import time
    t_total = 0.0
    extrap_steps = 0
    measured_steps = 0
    t_start = time.perf_counter()
    for op in layer_ops:
        if op[0] != 'truncate':
            t0 = time.perf_counter()
            if op[0] == '1q':
                apply_1q(st, op[1], op[2])
            else:
                i, t = orient_2q(op[1], op[2], op[3])
                apply_2q(st, i, t)
            t_total += time.perf_counter() - t0
            continue
        if not connected(st):
            continue
        t0 = time.perf_counter()
        qr_left2right(st)
        t_total += time.perf_counter() - t0
        step_t = {0: [], 1: []}
        for idx in range(st.n - 1, 0, -1):
            kind = idx % 2
            if time.perf_counter() - t_start > budget_s and step_t[kind]:
                t_total += sum(step_t[kind]) / len(step_t[kind])
                extrap_steps += 1
                # keep the shapes of the truncated sites (values are no longer
                # used for anything but timing)
                a, b = st.sites[idx - 1], st.sites[idx]
                k = min(chi or 10 ** 9, a.shape[0] * 2 * a.shape[2], 2 * b.shape[2] * b.shape[3])
                # (no exact-zero blocks: some LAPACK builds abort the process
                # on all-zero inputs)
                g = torch.Generator().manual_seed(idx)
                a2 = 1e-3 * torch.randn(a.shape[:3] + (k,), dtype=a.dtype, generator=g)
                b2 = 1e-3 * torch.randn((k,) + b.shape[1:], dtype=b.dtype, generator=g)
                kk = min(k, a.shape[3])
                a2[..., :kk] = a[..., :kk]
                b2[:kk] = b[:kk]
                st.sites[idx - 1], st.sites[idx] = a2, b2
                continue
            t0 = time.perf_counter()
            a, b = st.sites[idx - 1], st.sites[idx]
            l, x, aa, _ = a.shape
            _, y, cc, r = b.shape
            m = torch.einsum('lsam,mtcr->lsatcr', a, b).reshape(l * x * aa, y * cc * r)
            u, s, vh, _ = svd_truncate(m, chi, max_err, relative=True, randomized=randomized)
            ss = torch.sqrt(s).to(m.dtype)
            k = s.numel()
            st.sites[idx - 1] = (u * ss[None, :]).reshape(l, x, aa, k)
            st.sites[idx] = (ss[:, None] * vh).reshape(k, y, cc, r)
            dt = time.perf_counter() - t0
            step_t[kind].append(dt)
            t_total += dt
            measured_steps += 1
        if noisy:
            t0 = time.perf_counter()
            svd_kappa(st, kappa, max_err, randomized)
            t_total += time.perf_counter() - t0
    return t_total, dict(measured_svd_steps=measured_steps, extrapolated_svd_steps=extrap_steps)
