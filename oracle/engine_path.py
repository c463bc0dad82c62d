"""The GB300 engine's order of operations, restated in plain torch, for the
gradient study: can an adjoint differentiate the engine's own sequence and
still give the reference path's gradient?

TEST INFRASTRUCTURE ONLY; the product never imports it.

The engine (csrc/engine.cu) evaluates the reference's evolution
(``mpdo_oracle.evolve``) in a different but equivalent order:

* a two-qubit gate stays pending on its pair; when the next operation on the
  pair is a truncate() that runs, the gate is fused into the QR
  left-to-right sweep: the left site (with the previous R absorbed) is viewed
  as (b a) x (s m) and factored by QR, the site becomes I_2 (x) Q', and R'
  and the gate / Kraus mix move into the right site -- no SVD of theta, so
  the split's absolute cutoff (weight ~1e-8) is not applied.  Any other
  operation on the pair splits it as the reference does;
* the right-to-left SVD sweep decomposes only the right site of each pair
  (the left one is an isometry after the QR sweep, so SVD(A_{i-1} A_i) =
  A_{i-1} SVD(A_i)), keeping min(chi, rows of the pair, columns) values and
  padding with zeros beyond the site's own rank, as the reference's pair SVD
  returns them.

Differentiated with the gradient oracle's truncated SVD (``oracle.adjoint``),
which keeps the numerical rank, so the padded zero directions drop out.
"""
from __future__ import annotations

from typing import Dict, Optional

import torch

from . import mpdo_oracle as O


class EngineChain:
    """An MPDO with pending two-qubit gates, evolved in the engine's order."""

    def __init__(self, st: O.MPDO):
        self.st = st
        self.pend: Dict[int, torch.Tensor] = {}

    @property
    def n(self):
        return self.st.n

    # -- pending pairs -------------------------------------------------------
    def materialize(self, i: int) -> None:
        """csrc/engine.cu materialize_pair: the reference's split (Circuit.py:74-136)."""
        t = self.pend.pop(i, None)
        if t is not None:
            O.apply_2q(self.st, i, t)

    def materialize_all(self) -> None:
        for i in sorted(self.pend):
            self.materialize(i)

    def apply_1q(self, site: int, g: torch.Tensor) -> None:
        for j in (site - 1, site):
            self.materialize(j)
        O.apply_1q(self.st, site, g)

    def apply_2q(self, i: int, t: torch.Tensor) -> None:
        for j in (i - 1, i, i + 1):
            self.materialize(j)
        self.pend[i] = t if t.dim() == 5 else t.unsqueeze(-1)
        self.st.bonds[i] = True

    # -- truncate() ----------------------------------------------------------
    def _qr_sweep(self) -> None:
        st = self.st
        R = None
        for i in range(st.n - 1):
            if R is not None:
                st.sites[i] = torch.einsum('kl,lsar->ksar', R, st.sites[i])
                R = None
            a_i = st.sites[i]
            b, _, a, m = a_i.shape
            t = self.pend.pop(i, None)
            if t is not None:
                # fused pair: At[(b, a)][(s, m)] = QR; site i = I_2 (x) Q'
                At = a_i.permute(0, 2, 1, 3).reshape(b * a, 2 * m)
                Q, Rp = O._qr(At)
                kq = Q.shape[1]
                eye = torch.eye(2, dtype=Q.dtype)
                st.sites[i] = torch.einsum('st,bak->bsatk', eye, Q.reshape(b, a, kq)).reshape(b, 2, a, 2 * kq)
                # W[s][k][t][c][r] = sum_m R'[k][s m] A_{i+1}[m][t][c][r], then the gate / Kraus mix
                B = st.sites[i + 1]
                W = torch.einsum('ksm,mtcr->sktcr', Rp.reshape(kq, 2, m), B)
                Z = torch.einsum('xystq,sktcr->xkycqr', t.to(W.dtype), W)
                c, r, K = B.shape[2], B.shape[3], t.shape[-1]
                st.sites[i + 1] = Z.reshape(2 * kq, 2, c * K, r)
                continue
            l, x, aa, r = a_i.shape
            Q, R = O._qr(a_i.reshape(l * x * aa, r))
            st.sites[i] = Q.reshape(l, x, aa, Q.shape[1])
        if R is not None:
            st.sites[-1] = torch.einsum('kl,lsar->ksar', R, st.sites[-1])

    def _svd_sweep(self, chi: Optional[int], max_err: Optional[float]) -> None:
        st = self.st
        for idx in range(st.n - 1, 0, -1):
            P, S = st.sites[idx - 1], st.sites[idx]
            b, _, c, r = S.shape
            pl, _, pa, _ = P.shape
            rows_prev, Nc = pl * 2 * pa, 2 * c * r
            nsv = min(rows_prev, Nc)
            cap = min(chi, nsv) if chi else nsv
            u, s, vh, _ = O.svd_truncate(S.reshape(b, Nc), cap, max_err, relative=True)
            k = s.numel()
            ss = torch.sqrt(s).to(S.dtype)
            L, Rf = u * ss[None, :], ss[:, None] * vh
            if k < cap and max_err is None and not (S.requires_grad or P.requires_grad):
                # zero singular values up to the cap, as the reference's pair SVD returns them
                # (with an error rule, the rule itself drops the pair's trailing zeros)
                L = torch.cat([L, L.new_zeros(b, cap - k)], 1)
                Rf = torch.cat([Rf, Rf.new_zeros(cap - k, Nc)], 0)
                k = cap
            st.sites[idx - 1] = torch.einsum('lsab,bk->lsak', P, L)
            st.sites[idx] = Rf.reshape(k, 2, c, r)

    def truncate(self, chi, kappa, max_err, noisy) -> None:
        """csrc/engine.cu truncate_layer."""
        if not O.connected(self.st):
            return
        if chi is not None or max_err is not None:
            self._qr_sweep()
            self._svd_sweep(chi, max_err)
        if noisy:
            self.materialize_all()
            O.svd_kappa(self.st, kappa, max_err)


def evolve(st: O.MPDO, ops, chi=None, kappa=None, max_err=None, noisy=False) -> O.MPDO:
    """``mpdo_oracle.evolve`` in the engine's order; returns the final state
    with every pending pair materialised."""
    ch = EngineChain(st)
    last = None
    for op in ops:
        if op[0] == '1q':
            ch.apply_1q(op[1], op[2])
        elif op[0] == '2q':
            i, t = O.orient_2q(op[1], op[2], op[3])
            ch.apply_2q(i, t)
        elif op[0] == 'truncate':
            ch.truncate(chi, kappa, max_err, noisy)
        last = op[0]
    if noisy and last not in ('truncate', None):
        ch.materialize_all()
        O.svd_kappa(st, kappa, max_err)
    ch.materialize_all()
    return st
