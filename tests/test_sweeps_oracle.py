"""The oracle's sweeps (TNNOptimizer.py:87-161) on random chains, on the CPU:
without a cap they leave rho unchanged and give each bond min(rows, cols);
with a cap the per-bond discarded weight is the weight each split dropped,
and the mirror sweeps agree on a chain whose bonds need no truncation."""
import numpy as np
import pytest
import torch

from oracle import mpdo_oracle as O


def _chain(bonds, kraus, seed):
    g = np.random.default_rng(seed)
    sites = [torch.tensor(g.normal(size=(bonds[i], 2, a, bonds[i + 1])) +
                          1j * g.normal(size=(bonds[i], 2, a, bonds[i + 1]))) for i, a in enumerate(kraus)]
    return O.MPDO(sites, [True] * (len(sites) - 1))


BONDS = [1, 4, 9, 12, 7, 3, 1]
KRAUS = [2, 1, 3, 2, 1, 2]


@pytest.mark.parametrize('sweep', ['right2left', 'left2right'])
def test_uncapped_sweep_keeps_rho(sweep):
    st = _chain(BONDS, KRAUS, 1)
    rho = O.reduced_dm(st)
    if sweep == 'right2left':
        O.qr_left2right(st)
        disc = O.svd_right2left(st, None, None)
    else:
        disc = O.svd_left2right(st, None, None)
    assert max(disc) < 1e-28
    torch.testing.assert_close(O.reduced_dm(st), rho, rtol=0, atol=1e-10 * rho.abs().max().item())
    for a, b in zip(st.sites, st.sites[1:]):
        assert a.shape[3] == b.shape[0]


def test_capped_left2right_discards_what_each_split_drops():
    st = _chain(BONDS, KRAUS, 2)
    ref = st.clone()
    disc = O.svd_left2right(st, 3, None)
    assert all(s.shape[3] <= 3 for s in st.sites[:-1])
    # replay the first split by hand: its dropped weight over the pair's total
    a, b = ref.sites[0], ref.sites[1]
    m = torch.einsum('lsam,mtcr->lsatcr', a, b).reshape(a.shape[0] * 2 * a.shape[2], -1)
    s = torch.linalg.svdvals(m)
    assert abs(disc[0] - float((s[3:] ** 2).sum() / (s ** 2).sum())) < 1e-12
    assert 0 < min(d for d in disc if d > 0) and max(disc) < 1


def test_mirror_sweeps_agree_without_truncation():
    st = _chain(BONDS, KRAUS, 3)
    a, b = st.clone(), st.clone()
    O.qr_left2right(a)
    O.svd_right2left(a, None, None)
    O.svd_left2right(b, None, None)
    torch.testing.assert_close(O.reduced_dm(a), O.reduced_dm(b), rtol=0, atol=1e-9 * O.reduced_dm(a).abs().max().item())
